// Batched LU solves of systems of order <= 16 (see batched.cu).
#include "batched_kernels.cuh"

namespace mgb {

int batched_bucket_16_lu(int queue, const int32_t *list, BatchQueues *q,
                       const int32_t *n, const int64_t *offA,
                       const elem_t *A, const int64_t *offv,
                       const elem_t *b, elem_t *x, int32_t *status) {
  return launch_batched_queue<elem_t, 16, 4, 2>(queue, list, q, n, offA, A,
                                                   offv, b, x, status, kPivotEps,
                                                   batched_tune(0, 0).ctas_per_sm);
}

}  // namespace mgb
