/*
 * CPU oracle, kernel half: ADER-DG element update restated in plain C.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU path and the
 * CPU baseline that bench.py times; the product library never links it.
 * Compiled twice (REAL=double -> liboracle_f64.so, REAL=float -> liboracle_f32.so)
 * by oracle/Makefile.
 *
 * Every kernel restates a tensor expression of the reference:
 *   ader      codegen/kernels/aderdg.py:463-537 (derivative + Taylor expansion),
 *             driven as in src/Kernels/LinearCK/Time.cpp:65-140 (coeffs = integrate(0, dt)),
 *             with dQ(i) restricted to the first B(N-i) basis functions (aderdg.py:507-517)
 *   taylor    aderdg.py:531-536 derivativeTaylorExpansion / src/Kernels/LinearCK/Time.cpp:237-254
 *   local     aderdg.py:337-351 (volume) and :373-386 (localFlux), skipped on
 *             dynamic-rupture faces as in src/Kernels/LinearCK/Local.cpp:150-157
 *   neighbor  aderdg.py:414-428 (neighboringFlux(h, j, i)), executed with
 *             h = faceRelations[face][1], j = faceRelations[face][0] (src/Kernels/LinearCK/Neighbor.cpp:66-90)
 *
 * Memory layout (yateto column-major, as the reference): per cell a B x Nq tensor with
 * the basis index fastest, cell stride B*Nq; 9x9 operators column-major (q + 9 p);
 * derivative families dQ(i) packed back to back with leading dimension B(N-i).
 * Global matrices arrive dense column-major and are compressed to CSR here.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#ifndef REAL
#define REAL double
#endif
typedef REAL real;

#define NQ 9

typedef struct {
  int rows, cols, nnz;
  int* rowptr;
  int* col;
  real* val;
} csr_t;

static csr_t csr_from_dense(const double* a, int rows, int cols, int row_lim, int col_lim) {
  /* a is rows x cols; the CSR keeps rows < row_lim and columns < col_lim */
  csr_t m;
  m.rows = row_lim;
  m.cols = col_lim;
  m.rowptr = (int*)calloc((size_t)row_lim + 1, sizeof(int));
  int nnz = 0;
  for (int r = 0; r < row_lim; ++r)
    for (int c = 0; c < col_lim; ++c)
      if (a[r + (size_t)rows * c] != 0.0) ++nnz;
  m.nnz = nnz;
  m.col = (int*)malloc(sizeof(int) * (nnz ? nnz : 1));
  m.val = (real*)malloc(sizeof(real) * (nnz ? nnz : 1));
  int k = 0;
  for (int r = 0; r < row_lim; ++r) {
    m.rowptr[r] = k;
    for (int c = 0; c < col_lim; ++c)
      if (a[r + (size_t)rows * c] != 0.0) {
        m.col[k] = c;
        m.val[k] = (real)a[r + (size_t)rows * c];
        ++k;
      }
  }
  m.rowptr[row_lim] = k;
  return m;
}

static void csr_free(csr_t* m) {
  free(m->rowptr);
  free(m->col);
  free(m->val);
}

static int nb3(int n) { return n * (n + 1) * (n + 2) / 6; }
static int nb2(int n) { return n * (n + 1) / 2; }

/* out[r, q] (+)= sum_l A[r, l] x[l, q]; ld of out/x given; q over NQ */
static void csr_apply(const csr_t* a, const real* x, int ldx, real* out, int ldo, int accumulate) {
  for (int q = 0; q < NQ; ++q) {
    for (int r = 0; r < a->rows; ++r) {
      real s = 0;
      for (int k = a->rowptr[r]; k < a->rowptr[r + 1]; ++k) s += a->val[k] * x[a->col[k] + (size_t)ldx * q];
      if (accumulate)
        out[r + (size_t)ldo * q] += s;
      else
        out[r + (size_t)ldo * q] = s;
    }
  }
}

/* out[r, p] += sum_q x[r, q] S[q, p], S column-major 9x9 (zeros skipped) */
static void right_apply(const real* x, int ldx, int rows, const real* s, real* out, int ldo) {
  for (int p = 0; p < NQ; ++p)
    for (int q = 0; q < NQ; ++q) {
      real v = s[q + NQ * p];
      if (v == (real)0) continue;
      for (int r = 0; r < rows; ++r) out[r + (size_t)ldo * p] += x[r + (size_t)ldx * q] * v;
    }
}

/* Global matrix bundle, dense column-major doubles in this order:
 * kDivM[3] (BxB), kDivMT[3] (BxB, already negated), rDivM[4] (BxF), fMrT[4] (FxB), rT[4] (FxB), fP[3] (FxF). */
typedef struct {
  const double *kDivM[3], *kDivMT[3], *rDivM[4], *fMrT[4], *rT[4], *fP[3];
} gview_t;

static gview_t gview(const double* g, int order) {
  gview_t v;
  int B = nb3(order), F = nb2(order);
  const double* p = g;
  for (int i = 0; i < 3; ++i) { v.kDivM[i] = p; p += (size_t)B * B; }
  for (int i = 0; i < 3; ++i) { v.kDivMT[i] = p; p += (size_t)B * B; }
  for (int i = 0; i < 4; ++i) { v.rDivM[i] = p; p += (size_t)B * F; }
  for (int i = 0; i < 4; ++i) { v.fMrT[i] = p; p += (size_t)F * B; }
  for (int i = 0; i < 4; ++i) { v.rT[i] = p; p += (size_t)F * B; }
  for (int i = 0; i < 3; ++i) { v.fP[i] = p; p += (size_t)F * F; }
  return v;
}

int oracle_derivatives_size(int order) {
  int s = 0;
  for (int i = 0; i < order; ++i) s += nb3(order - i) * NQ;
  return s;
}

/* Cauchy-Kovalevskaya predictor: I = sum_i coeffs[i] dQ(i); optional derivative output. */
void oracle_ader(int order, int64_t ncells, const double* gmat, const real* Q, const real* star,
                 const double* coeffs, real* I, real* derivs) {
  const int B = nb3(order);
  gview_t g = gview(gmat, order);
  csr_t kt[8][3];
  for (int i = 1; i < order; ++i)
    for (int e = 0; e < 3; ++e)
      kt[i][e] = csr_from_dense(g.kDivMT[e], B, B, nb3(order - i), nb3(order - i + 1));
  const int dsz = oracle_derivatives_size(order);
#pragma omp parallel
  {
    real* dq = (real*)malloc(sizeof(real) * (size_t)dsz);
    real* tmp = (real*)malloc(sizeof(real) * (size_t)B * NQ);
#pragma omp for schedule(static)
    for (int64_t c = 0; c < ncells; ++c) {
      const real* q = Q + (size_t)c * B * NQ;
      real* out = I + (size_t)c * B * NQ;
      const real* st = star + (size_t)c * 3 * 81;
      memcpy(dq, q, sizeof(real) * (size_t)B * NQ);
      for (int k = 0; k < B * NQ; ++k) out[k] = (real)coeffs[0] * q[k];
      size_t off_prev = 0, off = (size_t)B * NQ;
      for (int i = 1; i < order; ++i) {
        const int bp = nb3(order - i + 1), bc = nb3(order - i);
        real* cur = dq + off;
        memset(cur, 0, sizeof(real) * (size_t)bc * NQ);
        for (int e = 0; e < 3; ++e) {
          memset(tmp, 0, sizeof(real) * (size_t)bc * NQ);
          csr_apply(&kt[i][e], dq + off_prev, bp, tmp, bc, 0);
          right_apply(tmp, bc, bc, st + 81 * e, cur, bc);
        }
        for (int p = 0; p < NQ; ++p)
          for (int k = 0; k < bc; ++k) out[k + (size_t)B * p] += (real)coeffs[i] * cur[k + (size_t)bc * p];
        off_prev = off;
        off += (size_t)bc * NQ;
      }
      if (derivs) memcpy(derivs + (size_t)c * dsz, dq, sizeof(real) * (size_t)dsz);
    }
    free(dq);
    free(tmp);
  }
  for (int i = 1; i < order; ++i)
    for (int e = 0; e < 3; ++e) csr_free(&kt[i][e]);
}

/* Taylor evaluation of packed derivatives: out = sum_i coeffs[i] dQ(i). */
void oracle_taylor(int order, int64_t ncells, const real* derivs, const double* coeffs, real* out) {
  const int B = nb3(order);
  const int dsz = oracle_derivatives_size(order);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < ncells; ++c) {
    const real* d = derivs + (size_t)c * dsz;
    real* o = out + (size_t)c * B * NQ;
    memset(o, 0, sizeof(real) * (size_t)B * NQ);
    size_t off = 0;
    for (int i = 0; i < order; ++i) {
      const int bi = nb3(order - i);
      for (int p = 0; p < NQ; ++p)
        for (int k = 0; k < bi; ++k) o[k + (size_t)B * p] += (real)coeffs[i] * d[off + k + (size_t)bi * p];
      off += (size_t)bi * NQ;
    }
  }
}

/* Volume + local flux: Q += sum_e kDivM_e I star_e + sum_{faces != DR} rDivM_f fMrT_f I AplusT_f. */
void oracle_local(int order, int64_t ncells, const double* gmat, const real* I, const real* star,
                  const real* aplus, const int8_t* face_type, real* Q) {
  const int B = nb3(order), F = nb2(order);
  gview_t g = gview(gmat, order);
  csr_t kd[3], rd[4], fm[4];
  for (int e = 0; e < 3; ++e) kd[e] = csr_from_dense(g.kDivM[e], B, B, B, B);
  for (int f = 0; f < 4; ++f) {
    rd[f] = csr_from_dense(g.rDivM[f], B, F, B, F);
    fm[f] = csr_from_dense(g.fMrT[f], F, B, F, B);
  }
#pragma omp parallel
  {
    real* tmp = (real*)malloc(sizeof(real) * (size_t)B * NQ);
    real* tf = (real*)malloc(sizeof(real) * (size_t)F * NQ);
    real* tf2 = (real*)malloc(sizeof(real) * (size_t)F * NQ);
#pragma omp for schedule(static)
    for (int64_t c = 0; c < ncells; ++c) {
      const real* in = I + (size_t)c * B * NQ;
      real* q = Q + (size_t)c * B * NQ;
      const real* st = star + (size_t)c * 3 * 81;
      for (int e = 0; e < 3; ++e) {
        csr_apply(&kd[e], in, B, tmp, B, 0);
        right_apply(tmp, B, B, st + 81 * e, q, B);
      }
      for (int f = 0; f < 4; ++f) {
        if (face_type && face_type[c * 4 + f] == 1) continue;
        csr_apply(&fm[f], in, B, tf, F, 0);
        memset(tf2, 0, sizeof(real) * (size_t)F * NQ);
        right_apply(tf, F, F, aplus + ((size_t)c * 4 + f) * 81, tf2, F);
        csr_apply(&rd[f], tf2, F, q, B, 1);
      }
    }
    free(tmp);
    free(tf);
    free(tf2);
  }
  for (int e = 0; e < 3; ++e) csr_free(&kd[e]);
  for (int f = 0; f < 4; ++f) {
    csr_free(&rd[f]);
    csr_free(&fm[f]);
  }
}

/* Neighbour flux on regular faces: Q += rDivM_i fP_h rT_j I_nb AminusT_i. */
void oracle_neighbor(int order, int64_t ncells, const double* gmat, const real* I, const real* aminus,
                     const int32_t* neighbor, const int8_t* side, const int8_t* orient,
                     const int8_t* face_type, real* Q) {
  const int B = nb3(order), F = nb2(order);
  gview_t g = gview(gmat, order);
  csr_t rd[4], rt[4], fp[3];
  for (int f = 0; f < 4; ++f) {
    rd[f] = csr_from_dense(g.rDivM[f], B, F, B, F);
    rt[f] = csr_from_dense(g.rT[f], F, B, F, B);
  }
  for (int h = 0; h < 3; ++h) fp[h] = csr_from_dense(g.fP[h], F, F, F, F);
#pragma omp parallel
  {
    real* t1 = (real*)malloc(sizeof(real) * (size_t)F * NQ);
    real* t2 = (real*)malloc(sizeof(real) * (size_t)F * NQ);
    real* t3 = (real*)malloc(sizeof(real) * (size_t)F * NQ);
#pragma omp for schedule(static)
    for (int64_t c = 0; c < ncells; ++c) {
      real* q = Q + (size_t)c * B * NQ;
      for (int f = 0; f < 4; ++f) {
        const size_t cf = (size_t)c * 4 + f;
        if (face_type && face_type[cf] != 0) continue;
        const int32_t nb = neighbor[cf];
        if (nb < 0) continue;
        const real* in = I + (size_t)nb * B * NQ;
        csr_apply(&rt[side[cf]], in, B, t1, F, 0);
        csr_apply(&fp[orient[cf]], t1, F, t2, F, 0);
        memset(t3, 0, sizeof(real) * (size_t)F * NQ);
        right_apply(t2, F, F, aminus + cf * 81, t3, F);
        csr_apply(&rd[f], t3, F, q, B, 1);
      }
    }
    free(t1);
    free(t2);
    free(t3);
  }
  for (int f = 0; f < 4; ++f) {
    csr_free(&rd[f]);
    csr_free(&rt[f]);
  }
  for (int h = 0; h < 3; ++h) csr_free(&fp[h]);
}

/* Proxy kernel 'all' for nsteps global time steps: per step ADER -> local, then neighbour
 * on the time-integrated DOFs of all cells (src/Proxy/KernelHost.cpp:108-198). */
void oracle_steps(int order, int64_t ncells, const double* gmat, real* Q, const real* star,
                  const real* aplus, const real* aminus, const int32_t* neighbor, const int8_t* side,
                  const int8_t* orient, const int8_t* face_type, const double* coeffs, int nsteps,
                  real* I_work) {
  for (int s = 0; s < nsteps; ++s) {
    oracle_ader(order, ncells, gmat, Q, star, coeffs, I_work, NULL);
    oracle_local(order, ncells, gmat, I_work, star, aplus, face_type, Q);
    oracle_neighbor(order, ncells, gmat, I_work, aminus, neighbor, side, orient, face_type, Q);
  }
}
