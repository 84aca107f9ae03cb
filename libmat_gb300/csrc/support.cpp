// Host-memory helpers of the mat.h API: construction, copies, element access,
// printing and comparison (mat.h:1266-1545, 2923-2930).  These manage the
// caller's host matrices exactly as the reference's do; they are not part of
// the compute path, which runs on the GPU (api.cu).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mat.h"

extern "C" {

Mat *mat_empty(size_t rows, size_t cols) {  // mat.h:1266-1275
  MAT_ASSERT_DIM(rows, cols);
  Mat *m = (Mat *)malloc(sizeof(Mat));
  m->rows = rows;
  m->cols = cols;
  m->data = NULL;
  return m;
}

Mat *mat_mat(size_t rows, size_t cols) {  // mat.h:1277-1282
  Mat *m = mat_empty(rows, cols);
  m->data = (mat_elem_t *)calloc(rows * cols, sizeof(mat_elem_t));
  return m;
}

void mat_init(Mat *out, const mat_elem_t *values) {  // mat.h:1293-1304
  MAT_ASSERT_MAT(out);
  MAT_ASSERT(values != NULL);
  for (size_t i = 0; i < out->rows; i++)
    for (size_t j = 0; j < out->cols; j++)
      MAT_SET(out, i, j, values[i * out->cols + j]);  // row-major input
}

Mat *mat_from(size_t rows, size_t cols, const mat_elem_t *values) {
  MAT_ASSERT_DIM(rows, cols);
  Mat *m = mat_mat(rows, cols);
  mat_init(m, values);
  return m;
}

void mat_free_mat(Mat *m) {
  MAT_ASSERT_MAT(m);
  MAT_FREE_MAT(m);
}

Mat *mat_zeros(size_t rows, size_t cols) { return mat_mat(rows, cols); }

void mat_fill(Mat *out, mat_elem_t value) {  // mat.h:1323-1330
  MAT_ASSERT_MAT(out);
  MAT_ASSERT(value >= 0);
  size_t len = out->rows * out->cols;
  for (size_t i = 0; i < len; i++) out->data[i] = value;
}

Mat *mat_ones(size_t rows, size_t cols) {
  MAT_ASSERT_DIM(rows, cols);
  Mat *m = mat_mat(rows, cols);
  mat_fill(m, (mat_elem_t)1.0);
  return m;
}

void mat_eye(Mat *out) {  // mat.h:1332-1340
  MAT_ASSERT_SQUARE(out);
  size_t d = out->rows;
  memset(out->data, 0, d * d * sizeof(mat_elem_t));
  for (size_t i = 0; i < d; i++) MAT_SET(out, i, i, 1);
}

Mat *mat_reye(size_t dim) {
  MAT_ASSERT(dim > 0);
  Mat *m = mat_mat(dim, dim);
  for (size_t i = 0; i < dim; i++) MAT_SET(m, i, i, 1);
  return m;
}

Vec *mat_vec(size_t dim) { return mat_mat(dim, 1); }
Vec *mat_row_vec(size_t dim) { return mat_mat(1, dim); }
Vec *mat_vec_from(size_t dim, const mat_elem_t *values) {
  return mat_from(dim, 1, values);
}

Perm *mat_perm(size_t n) {  // mat.h:1369-1374
  Perm *p = (Perm *)malloc(sizeof(Perm));
  p->data = (size_t *)malloc(n * sizeof(size_t));
  p->size = n;
  return p;
}

void mat_free_perm(Perm *p) {
  free(p->data);
  free(p);
}

void mat_perm_identity(Perm *p) {
  for (size_t i = 0; i < p->size; i++) p->data[i] = i;
}

Mat *mat_perm_mat(const Perm *p) {  // mat.h:1387-1394: row i has a 1 at p[i]
  size_t n = p->size;
  Mat *m = mat_zeros(n, n);
  for (size_t i = 0; i < n; i++) MAT_SET(m, i, p->data[i], 1);
  return m;
}

// The reference's mat_copy returns a new zero-filled matrix of the same shape
// (mat.h:1396-1402); kept as is so callers see the same behaviour.
Mat *mat_copy(const Mat *m) {
  MAT_ASSERT_MAT(m);
  return mat_mat(m->rows, m->cols);
}

void mat_deep_copy(Mat *out, const Mat *src) {
  MAT_ASSERT_MAT(out);
  MAT_ASSERT_MAT(src);
  MAT_ASSERT(out->rows == src->rows && out->cols == src->cols);
  memcpy(out->data, src->data, src->rows * src->cols * sizeof(mat_elem_t));
}

Mat *mat_rdeep_copy(const Mat *m) {
  MAT_ASSERT_MAT(m);
  Mat *r = mat_copy(m);
  memcpy(r->data, m->data, m->rows * m->cols * sizeof(mat_elem_t));
  return r;
}

mat_elem_t mat_at(const Mat *m, size_t row, size_t col) {
  MAT_ASSERT_MAT(m);
  return MAT_AT(m, row, col);
}

void mat_set_at(Mat *m, size_t row, size_t col, mat_elem_t value) {
  MAT_ASSERT_MAT(m);
  MAT_SET(m, row, col, value);
}

MatSize mat_size(const Mat *m) {
  MatSize s = {m->rows, m->cols};
  return s;
}

void mat_print(const Mat *mat) {  // mat.h:1441-1462
  MAT_ASSERT(mat != NULL);
  MAT_ASSERT(mat->data != NULL);
  printf("[");
  for (size_t i = 0; i < mat->rows; i++) {
    if (i > 0) printf(" ");
    for (size_t j = 0; j < mat->cols; j++) {
      printf("%g", (double)MAT_AT(mat, i, j));
      if (j < mat->cols - 1) printf(" ");
    }
    if (i < mat->rows - 1) printf(";\n");
  }
  printf("]\n");
}

// Absolute element-wise comparison (mat.h:1521-1545).
bool mat_equals_tol(const Mat *a, const Mat *b, mat_elem_t epsilon) {
  MAT_ASSERT_MAT(a);
  MAT_ASSERT_MAT(b);
  if (a->rows != b->rows || a->cols != b->cols) return false;
  size_t n = a->rows * a->cols;
  for (size_t i = 0; i < n; i++) {
    mat_elem_t d = a->data[i] - b->data[i];
    if (d < 0) d = -d;
    if (d > epsilon) return false;
  }
  return true;
}

bool mat_equals(const Mat *a, const Mat *b) {
  return mat_equals_tol(a, b, MAT_DEFAULT_EPSILON);
}

Mat *mat_rt(const Mat *m) {  // mat.h:2923-2930 (transpose into a new matrix)
  MAT_ASSERT_MAT(m);
  Mat *r = mat_mat(m->cols, m->rows);
  for (size_t j = 0; j < m->cols; j++)
    for (size_t i = 0; i < m->rows; i++) MAT_SET(r, j, i, MAT_AT(m, i, j));
  return r;
}

}  // extern "C"
