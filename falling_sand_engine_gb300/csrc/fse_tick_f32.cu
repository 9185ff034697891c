// fse_tick_f32.cu -- the colour pass of worlds with f32 liquid amounts
// (FSE_CFG_F32_FLUID) in the partitioned order: the F32 instantiations of
// fse_tick.cu's kernel, built as their own translation unit so that they compile in
// parallel with the others.
#define FSE_TICK_F32_TU 1
#include "fse_tick.cu"
