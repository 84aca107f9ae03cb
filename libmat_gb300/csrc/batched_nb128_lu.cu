// Batched LU solves of systems of order <= 128 (see batched.cu): the
// blocked LU kernel (batched_blk.cuh) or the register Gauss-Jordan kernel
// (batched_kernels.cuh), as the tuning table picks.
#include "batched_smem.cuh"

namespace mgb {

int batched_bucket_128_lu(int queue, const int32_t *list, BatchQueues *q,
                          const int32_t *n, const int64_t *offA,
                          const elem_t *A, const int64_t *offv,
                          const elem_t *b, elem_t *x, int32_t *status) {
  const BatchTune &t = batched_tune(4, 0);
#ifdef MAT_DOUBLE_PRECISION
  // a row of this order does not fit in registers in double precision: the
  // rows live in shared memory (batched_smem.cuh)
  (void)t;
  return launch_smem_queue<elem_t, 128, 0>(queue, list, q, n, offA, A, offv, b, x,
                                              status, kPivotEps);
#else
  if (t.algo == 1)
    return launch_blk_queue<elem_t, 128, 0, 2>(queue, list, q, n, offA, A, offv,
                                                   b, x, status, kPivotEps, t.ctas_per_sm);
  return launch_batched_queue<elem_t, 128, 1, 2>(queue, list, q, n, offA, A,
                                                   offv, b, x, status, kPivotEps,
                                                   t.ctas_per_sm);
#endif
}

}  // namespace mgb
