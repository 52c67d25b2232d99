// Fast variant of the ACM stage kernel: the convective form uses the
// regrouped stencil algebra of rhs_opt, the skew-symmetric form the
// reference's expressions with FMA contraction (results agree with the
// reference to a few ulp per stage).
#define WG_NS fast
#define WG_FAST_ALGEBRA 1
#include "acm_body.cuh"
