// fse_tick_pair_f32.cu -- the colour pass with each chunk split over a CTA pair (a thread-block
// cluster of two), f32 liquid amounts (FSE_CFG_F32_FLUID): the PAIR instantiations of fse_tick.cu's kernel,
// built as their own translation unit so that they compile in parallel with the others.
#define FSE_TICK_PAIR_TU 2
#include "fse_tick.cu"
