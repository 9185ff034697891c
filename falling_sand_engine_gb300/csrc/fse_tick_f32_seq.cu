// fse_tick_f32_seq.cu -- the colour pass of worlds with f32 liquid amounts
// (FSE_CFG_F32_FLUID) in the reference's own order (FSE_CFG_REFERENCE_ORDER): the
// F32 SEQ instantiations of fse_tick.cu's kernel, in a translation unit of their own.
#define FSE_TICK_F32_TU 2
#include "fse_tick.cu"
