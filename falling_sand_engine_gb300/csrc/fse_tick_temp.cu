// fse_tick_temp.cu -- the colour pass of worlds that keep liquid temperatures
// (FSE_CFG_TEMPERATURE): the TEMP instantiation of fse_tick.cu's kernel, built as
// its own translation unit so that both instantiations compile in parallel.
#define FSE_TICK_TEMP_TU 1
#include "fse_tick.cu"
