// Batched LU solves of systems of order <= 96 (see batched.cu).
#include "batched_kernels.cuh"

namespace mgb {

int batched_bucket_96_lu(int queue, const int32_t *list, BatchQueues *q,
                       const int32_t *n, const int64_t *offA,
                       const elem_t *A, const int64_t *offv,
                       const elem_t *b, elem_t *x, int32_t *status) {
#ifdef MAT_DOUBLE_PRECISION
  // A row of this order does not fit in registers in double precision; the
  // driver has marked these systems with status -2.
  (void)queue; (void)list; (void)q; (void)n; (void)offA; (void)A; (void)offv;
  (void)b; (void)x; (void)status;
  return 0;
#else
  return launch_batched_queue<elem_t, 96, 1, 2>(queue, list, q, n, offA, A,
                                                   offv, b, x, status, kPivotEps);
#endif
}

}  // namespace mgb
