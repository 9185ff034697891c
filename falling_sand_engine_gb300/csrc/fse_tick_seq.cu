// fse_tick_seq.cu -- the colour pass in the reference's own order inside each chunk
// (FSE_CFG_REFERENCE_ORDER): the SEQ instantiations of fse_tick.cu's kernel, built
// as their own translation unit so that they compile in parallel with the others.
#define FSE_TICK_SEQ_TU 1
#include "fse_tick.cu"
