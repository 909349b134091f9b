// Mixed-precision grand-resistance solve (FP32 factorisations with FP64
// refinement).  Built in a later step; the fused step refuses the mode.
#include "rsd_internal.cuh"
