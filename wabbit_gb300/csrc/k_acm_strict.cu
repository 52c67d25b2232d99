// Strict variant of the ACM stage kernel: compiled with -fmad=false so every
// multiply and add rounds separately, in the reference's order (bit-identical
// to the reference's FD_4th_central RHS and RK4 update).
#define WG_NS strict
#include "acm_body.cuh"
