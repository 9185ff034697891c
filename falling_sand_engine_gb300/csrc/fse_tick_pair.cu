// fse_tick_pair.cu -- the colour pass with each chunk split over a CTA pair (a thread-block
// cluster of two), Q16.16 liquid amounts: the PAIR instantiations of fse_tick.cu's kernel,
// built as their own translation unit so that they compile in parallel with the others.
#define FSE_TICK_PAIR_TU 1
#include "fse_tick.cu"
