// fse_tick_fused.cu -- the fused tick (every colour pass of a tick in one launch,
// chunk-passes started as the chunk-passes they depend on finish) for Q16.16
// liquid amounts: fse_tick.cu's kernel with FUSED, built as its own translation
// unit so that it compiles in parallel with the others.
#define FSE_TICK_FUSED_TU 1
#include "fse_tick.cu"
