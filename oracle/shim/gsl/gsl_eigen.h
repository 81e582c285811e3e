/*
 * Stand-in for the part of GSL's symmetric eigensolver API that the reference
 * calls (External/matvec.h Eig, used by Functions.cpp Rotation for the 3D
 * tensile-instability rotation). Written for this project: a cyclic Jacobi
 * iteration on a dense symmetric matrix (Golub & Van Loan, "Matrix
 * Computations", sec. 8.5), not GSL's QR-based code. Eigenvalues agree with any
 * correct solver to rounding; the 3D TI tensor R diag(.) R^T it feeds is
 * invariant to eigenvector sign and to the order of equal eigenvalues.
 * TEST INFRASTRUCTURE ONLY.
 */
#ifndef PSPH_SHIM_GSL_EIGEN_H
#define PSPH_SHIM_GSL_EIGEN_H

#include <cmath>
#include <cstddef>
#include <cstdlib>

typedef struct {
  size_t size;
  size_t stride;
  double* data;
  void* block;
  int owner;
} gsl_vector;

typedef struct {
  size_t size1;
  size_t size2;
  size_t tda;
  double* data;
  void* block;
  int owner;
} gsl_matrix;

typedef struct {
  gsl_matrix matrix;
} gsl_matrix_view;

typedef struct {
  gsl_vector vector;
} gsl_vector_view;

typedef struct {
  size_t n;
} gsl_eigen_symm_workspace;
typedef gsl_eigen_symm_workspace gsl_eigen_symmv_workspace;

typedef enum { GSL_EIGEN_SORT_VAL_ASC, GSL_EIGEN_SORT_VAL_DESC, GSL_EIGEN_SORT_ABS_ASC, GSL_EIGEN_SORT_ABS_DESC } gsl_eigen_sort_t;

static inline gsl_matrix_view gsl_matrix_view_array(double* base, size_t n1, size_t n2) {
  gsl_matrix_view v;
  v.matrix.size1 = n1;
  v.matrix.size2 = n2;
  v.matrix.tda = n2;
  v.matrix.data = base;
  v.matrix.block = NULL;
  v.matrix.owner = 0;
  return v;
}

static inline gsl_vector* gsl_vector_alloc(size_t n) {
  gsl_vector* v = (gsl_vector*)std::malloc(sizeof(gsl_vector));
  v->size = n;
  v->stride = 1;
  v->data = (double*)std::calloc(n, sizeof(double));
  v->block = NULL;
  v->owner = 1;
  return v;
}
static inline void gsl_vector_free(gsl_vector* v) {
  if (!v) return;
  if (v->owner) std::free(v->data);
  std::free(v);
}
static inline gsl_matrix* gsl_matrix_alloc(size_t n1, size_t n2) {
  gsl_matrix* m = (gsl_matrix*)std::malloc(sizeof(gsl_matrix));
  m->size1 = n1;
  m->size2 = n2;
  m->tda = n2;
  m->data = (double*)std::calloc(n1 * n2, sizeof(double));
  m->block = NULL;
  m->owner = 1;
  return m;
}
static inline void gsl_matrix_free(gsl_matrix* m) {
  if (!m) return;
  if (m->owner) std::free(m->data);
  std::free(m);
}
static inline double gsl_vector_get(const gsl_vector* v, size_t i) { return v->data[i * v->stride]; }
static inline gsl_vector_view gsl_matrix_column(gsl_matrix* m, size_t j) {
  gsl_vector_view v;
  v.vector.size = m->size1;
  v.vector.stride = m->tda;
  v.vector.data = m->data + j;
  v.vector.block = NULL;
  v.vector.owner = 0;
  return v;
}

static inline gsl_eigen_symm_workspace* gsl_eigen_symm_alloc(size_t n) {
  gsl_eigen_symm_workspace* w = (gsl_eigen_symm_workspace*)std::malloc(sizeof(gsl_eigen_symm_workspace));
  w->n = n;
  return w;
}
static inline void gsl_eigen_symm_free(gsl_eigen_symm_workspace* w) { std::free(w); }
static inline gsl_eigen_symmv_workspace* gsl_eigen_symmv_alloc(size_t n) { return gsl_eigen_symm_alloc(n); }
static inline void gsl_eigen_symmv_free(gsl_eigen_symmv_workspace* w) { std::free(w); }

/* Cyclic Jacobi: A (symmetric, overwritten) -> eigenvalues in eval, eigenvectors
 * in the columns of evec (may be NULL). */
static inline int psph_shim_jacobi(gsl_matrix* A, gsl_vector* eval, gsl_matrix* evec) {
  const size_t n = A->size1;
  double* a = (double*)std::malloc(n * n * sizeof(double));
  double* q = (double*)std::malloc(n * n * sizeof(double));
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < n; ++j) {
      a[i * n + j] = A->data[i * A->tda + j];
      q[i * n + j] = (i == j) ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (size_t i = 0; i < n; ++i)
      for (size_t j = i + 1; j < n; ++j) off += a[i * n + j] * a[i * n + j];
    if (off == 0.0) break;
    for (size_t p = 0; p < n; ++p)
      for (size_t r = p + 1; r < n; ++r) {
        const double apr = a[p * n + r];
        if (apr == 0.0) continue;
        const double theta = (a[r * n + r] - a[p * n + p]) / (2.0 * apr);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0);
        const double s = t * c;
        for (size_t k = 0; k < n; ++k) {  // A <- A J (columns p, r)
          const double akp = a[k * n + p], akr = a[k * n + r];
          a[k * n + p] = c * akp - s * akr;
          a[k * n + r] = s * akp + c * akr;
        }
        for (size_t k = 0; k < n; ++k) {  // A <- J^T A (rows p, r)
          const double apk = a[p * n + k], ark = a[r * n + k];
          a[p * n + k] = c * apk - s * ark;
          a[r * n + k] = s * apk + c * ark;
        }
        for (size_t k = 0; k < n; ++k) {  // Q <- Q J
          const double qkp = q[k * n + p], qkr = q[k * n + r];
          q[k * n + p] = c * qkp - s * qkr;
          q[k * n + r] = s * qkp + c * qkr;
        }
      }
  }
  for (size_t i = 0; i < n; ++i) eval->data[i * eval->stride] = a[i * n + i];
  if (evec)
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j < n; ++j) evec->data[i * evec->tda + j] = q[i * n + j];
  std::free(a);
  std::free(q);
  return 0;
}

static inline int gsl_eigen_symm(gsl_matrix* A, gsl_vector* eval, gsl_eigen_symm_workspace*) {
  return psph_shim_jacobi(A, eval, NULL);
}
static inline int gsl_eigen_symmv(gsl_matrix* A, gsl_vector* eval, gsl_matrix* evec, gsl_eigen_symmv_workspace*) {
  return psph_shim_jacobi(A, eval, evec);
}

/* Selection sort of eigenvalues, permuting eigenvector columns alongside. */
static inline int gsl_eigen_symmv_sort(gsl_vector* eval, gsl_matrix* evec, gsl_eigen_sort_t type) {
  const size_t n = eval->size;
  for (size_t i = 0; i + 1 < n; ++i) {
    size_t best = i;
    for (size_t j = i + 1; j < n; ++j) {
      const double vj = eval->data[j * eval->stride], vb = eval->data[best * eval->stride];
      bool better = false;
      switch (type) {
        case GSL_EIGEN_SORT_VAL_ASC: better = vj < vb; break;
        case GSL_EIGEN_SORT_VAL_DESC: better = vj > vb; break;
        case GSL_EIGEN_SORT_ABS_ASC: better = std::fabs(vj) < std::fabs(vb); break;
        case GSL_EIGEN_SORT_ABS_DESC: better = std::fabs(vj) > std::fabs(vb); break;
      }
      if (better) best = j;
    }
    if (best != i) {
      double t = eval->data[i * eval->stride];
      eval->data[i * eval->stride] = eval->data[best * eval->stride];
      eval->data[best * eval->stride] = t;
      for (size_t k = 0; k < evec->size1; ++k) {
        double u = evec->data[k * evec->tda + i];
        evec->data[k * evec->tda + i] = evec->data[k * evec->tda + best];
        evec->data[k * evec->tda + best] = u;
      }
    }
  }
  return 0;
}

#endif
