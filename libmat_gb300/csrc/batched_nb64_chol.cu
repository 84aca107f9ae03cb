// Batched Cholesky solves of systems of order <= 64 (see batched.cu): the
// blocked LU kernel (batched_blk.cuh) or the register Gauss-Jordan kernel
// (batched_kernels.cuh), as the tuning table picks.
#include "batched_blk.cuh"

namespace mgb {

int batched_bucket_64_chol(int queue, const int32_t *list, BatchQueues *q,
                           const int32_t *n, const int64_t *offA,
                           const elem_t *A, const int64_t *offv,
                           const elem_t *b, elem_t *x, int32_t *status) {
  const BatchTune &t = batched_tune(2, 1);
  if (t.algo == 1)
    return launch_blk_queue<elem_t, 64, 1, (sizeof(elem_t) == 8 ? 3 : 5)>(queue, list, q, n, offA, A, offv,
                                                   b, x, status, kPivotEps, t.ctas_per_sm);
  return launch_batched_queue<elem_t, 64, 1, 1>(queue, list, q, n, offA, A,
                                                   offv, b, x, status, kPivotEps,
                                                   t.ctas_per_sm);
}

}  // namespace mgb
