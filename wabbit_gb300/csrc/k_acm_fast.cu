// Fast variant of the ACM stage kernel: same expressions as the strict one,
// compiled with FMA contraction (results agree with the reference to a few
// ulp per stage).
#define WG_NS fast
#include "acm_body.cuh"
