// k_fused_final.cu -- the final stage's launcher and its kernel instantiations (three tile
// shapes of every form), compiled apart from k_fused.cu so that the two heaviest sets of
// kernels build in parallel.
#define GLS_FUSED_FINAL_TU
#include "k_fused.cu"
