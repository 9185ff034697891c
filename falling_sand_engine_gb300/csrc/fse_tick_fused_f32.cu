// fse_tick_fused_f32.cu -- the fused tick for worlds with f32 liquid amounts
// (FSE_CFG_F32_FLUID): fse_tick.cu's kernel with FUSED and F32, built as its own
// translation unit so that it compiles in parallel with the others.
#define FSE_TICK_FUSED_TU 2
#include "fse_tick.cu"
