/*
 * nl_oracle.c -- CPU restatement of NeighbourLists.jl (v0.6.2) for testing.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle for the
 * GPU neighbour-list engine.  Only the test suite, the smoke check and the
 * CPU-baseline leg of the benchmark may load it; the product never calls it.
 *
 * What is restated (file:line are paths inside the reference project):
 *   - cell-index algebra            src/cell_list.jl:30-170
 *   - 3x3 inv/det/cross/norm in the operation order of StaticArrays.jl 1.x
 *     (a third-party dependency, compat "1", not vendored and not pinned by
 *     a Manifest; the order used here is the unrolled left-to-right form of
 *     its generated 3x3 methods)
 *   - sort-based CPU build          src/cell_list.jl:632-750
 *   - shared traversal              src/gpu_kernels.jl:20-101
 *   - count / offsets / fill        src/gpu_kernels.jl:132-180,199-237,299-364
 *   - pair vector R (_getR)         src/cell_list.jl:525-531
 *   - lazy traversal                src/cell_list.jl:779-833
 *   - legacy linked-list PairList   src/cell_list.jl:172-505
 *
 * Floating point: Julia never contracts a*b+c into an FMA unless asked to,
 * so this file must be compiled with -ffp-contract=off (the Makefile does).
 * Every mat-vec is a left fold ((a1*b1 + a2*b2) + a3*b3), as StaticArrays'
 * unrolled `_mul` and `_vecdot` generate it.
 *
 * Index conventions: all index outputs are 1-based like the reference.
 * Matrices are 9 doubles in column-major order (Julia SMatrix layout):
 * M[r + 3*c] is row r, column c; the rows of the cell are lattice vectors.
 * Integers are carried as int64; the index type TI of the reference only
 * enters through its overflow checks (ti_bytes = 4 for Int32, 8 for Int64).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_ERR_ARG 1
#define ORC_ERR_TOO_MANY_CELLS 2
#define ORC_ERR_NOMEM 3

/* ------------------------------------------------------------------ */
/* StaticArrays-style 3-vector / 3x3 helpers                           */
/* ------------------------------------------------------------------ */

static void sa_cross(const double a[3], const double b[3], double o[3]) {
  /* cross(a,b) = (a2 b3 - a3 b2, a3 b1 - a1 b3, a1 b2 - a2 b1) */
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

static double sa_dot(const double a[3], const double b[3]) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

static double sa_norm(const double a[3]) { return sqrt((a[0] * a[0] + a[1] * a[1]) + a[2] * a[2]); }

/* det: first column dotted with cross(second column, third column) */
static double sa_det(const double M[9]) {
  double c[3];
  sa_cross(M + 3, M + 6, c);
  return sa_dot(M, c);
}

/* inv: y0 = x1 x x2; d = x0.y0; x0/=d; y0/=d; y1 = x2 x x0; y2 = x0 x x1;
 * result rows are y0, y1, y2 (x0,x1,x2 = columns of M). */
static void sa_inv(const double M[9], double out[9]) {
  double x0[3] = {M[0], M[1], M[2]}, x1[3] = {M[3], M[4], M[5]}, x2[3] = {M[6], M[7], M[8]};
  double y0[3], y1[3], y2[3];
  sa_cross(x1, x2, y0);
  double d = sa_dot(x0, y0);
  for (int k = 0; k < 3; ++k) {
    x0[k] = x0[k] / d;
    y0[k] = y0[k] / d;
  }
  sa_cross(x2, x0, y1);
  sa_cross(x0, x1, y2);
  for (int c = 0; c < 3; ++c) {
    out[0 + 3 * c] = y0[c];
    out[1 + 3 * c] = y1[c];
    out[2 + 3 * c] = y2[c];
  }
}

static void row_of(const double M[9], int r, double v[3]) {
  v[0] = M[r];
  v[1] = M[r + 3];
  v[2] = M[r + 6];
}

/* M' * v for double v:  component k = sum_m M[m,k] v[m]  (left fold) */
static void matT_vec(const double M[9], const double v[3], double o[3]) {
  for (int k = 0; k < 3; ++k) o[k] = (M[0 + 3 * k] * v[0] + M[1 + 3 * k] * v[1]) + M[2 + 3 * k] * v[2];
}

/* M * v : component r = sum_k M[r,k] v[k] (left fold) */
static void mat_vec(const double M[9], const double v[3], double o[3]) {
  for (int r = 0; r < 3; ++r) o[r] = (M[r + 0] * v[0] + M[r + 3] * v[1]) + M[r + 6] * v[2];
}

/* ------------------------------------------------------------------ */
/* cell_list.jl:94-95 lengths, :152-170 analyze_cell,                  */
/* gpu_kernels.jl:315-316 nxyz                                         */
/* ------------------------------------------------------------------ */

void orc_lengths(const double C[9], double lens[3]) {
  double r1[3], r2[3], r3[3], c[3];
  row_of(C, 0, r1);
  row_of(C, 1, r2);
  row_of(C, 2, r3);
  double det = sa_det(C);
  double n[3];
  sa_cross(r2, r3, c);
  n[0] = sa_norm(c);
  sa_cross(r3, r1, c);
  n[1] = sa_norm(c);
  sa_cross(r1, r2, c);
  n[2] = sa_norm(c);
  for (int k = 0; k < 3; ++k) lens[k] = det / n[k];
}

int orc_analyze_cell(const double C[9], double cutoff, int ti_bytes, double inv_cell[9], int64_t ns[3],
                     double lens[3], int64_t nxyz[3]) {
  if (!(cutoff > 0)) return ORC_ERR_ARG;
  sa_inv(C, inv_cell);
  orc_lengths(C, lens);
  double tmax = ti_bytes == 4 ? 2147483647.0 : 9223372036854775807.0;
  long double prod = 1;
  for (int k = 0; k < 3; ++k) {
    lens[k] = fabs(lens[k]);
    double t = floor(lens[k] / cutoff);
    if (!(t < tmax)) return ORC_ERR_TOO_MANY_CELLS; /* floor(TI, .) InexactError */
    ns[k] = t < 1 ? 1 : (int64_t)t;
    prod *= (long double)ns[k];
  }
  if (prod > (long double)tmax) return ORC_ERR_TOO_MANY_CELLS; /* cell_list.jl:655-659 */
  for (int k = 0; k < 3; ++k) nxyz[k] = (int64_t)ceil(cutoff * ((double)ns[k] / lens[k]));
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* cell index algebra, cell_list.jl:33-147                             */
/* ------------------------------------------------------------------ */

/* position_to_cell_index: frac = inv' x ; c = floor(frac*n + 1) */
static void p2c(const double inv[9], const double x[3], const int64_t ns[3], int64_t c[3]) {
  double f[3];
  matT_vec(inv, x, f);
  for (int k = 0; k < 3; ++k) c[k] = (int64_t)floor(f[k] * (double)ns[k] + 1.0);
}

static int64_t bin_wrap(int64_t i, int64_t n) {
  /* while i <= 0: i += n; while i > n: i -= n  (closed form) */
  if (i <= 0) i += ((-i) / n + 1) * n;
  if (i > n) i -= ((i - 1) / n) * n;
  return i;
}

static int64_t clampi(int64_t i, int64_t lo, int64_t hi) { return i < lo ? lo : (i > hi ? hi : i); }

/* wrap_and_shift: returns wrapped index, shift s with i == wrapped + s*n */
static int64_t wrap_and_shift(int64_t i, int64_t n, int pbc, int64_t* s) {
  if (!pbc) {
    *s = 0;
    return clampi(i, 1, n);
  }
  int64_t w = bin_wrap(i, n);
  *s = (i - w) / n;
  return w;
}

static int64_t sub2ind(const int64_t ns[3], const int64_t c[3]) {
  return c[0] + (c[1] - 1) * ns[0] + (c[2] - 1) * ns[0] * ns[1];
}

/* ------------------------------------------------------------------ */
/* sort-based CPU build, cell_list.jl:647-748                          */
/* ------------------------------------------------------------------ */

typedef struct {
  const double* X; /* original positions, nat x 3 */
  int64_t nat;
  double C[9], inv[9], lens[3], cutoff, cutoff_sq;
  int64_t ns[3], nxyz[3], ncells;
  uint8_t pbc[3];
  const int64_t* perm;         /* 1-based, length nat */
  const int64_t* cell_offsets; /* 1-based, length ncells+1 */
} orc_clist;

/* Builds the sorted cell list.  perm/cell_id_sorted/X_sorted: length nat;
 * cell_offsets: length ncells+1 (ncells from orc_analyze_cell). */
int orc_build_cell_list(const double* X, int64_t nat, const double C[9], const uint8_t pbc[3], double cutoff,
                        int ti_bytes, int64_t* perm, int64_t* cell_id_sorted, int64_t* cell_offsets,
                        double* X_sorted) {
  double inv[9], lens[3];
  int64_t ns[3], nxyz[3];
  int st = orc_analyze_cell(C, cutoff, ti_bytes, inv, ns, lens, nxyz);
  if (st) return st;
  int64_t ncells = ns[0] * ns[1] * ns[2];
  int64_t* cid = (int64_t*)malloc(sizeof(int64_t) * (nat > 0 ? nat : 1));
  if (!cid) return ORC_ERR_NOMEM;
  /* _compute_cell_ids (CPU): bin_wrap_or_trunc then _sub2ind, :684-701 */
  for (int64_t i = 0; i < nat; ++i) {
    int64_t c[3];
    p2c(inv, X + 3 * i, ns, c);
    for (int k = 0; k < 3; ++k) c[k] = pbc[k] ? bin_wrap(c[k], ns[k]) : clampi(c[k], 1, ns[k]);
    cid[i] = sub2ind(ns, c);
  }
  /* stable sortperm (Base.sortperm is stable) -- a stable counting sort, :706-708 */
  for (int64_t c = 0; c <= ncells; ++c) cell_offsets[c] = 0;
  for (int64_t i = 0; i < nat; ++i) cell_offsets[cid[i]] += 1; /* counts at index cid (1-based slot) */
  /* _compute_cell_offsets, :724-748: offsets[1] = 1; offsets[c+1] += offsets[c] */
  if (nat == 0) {
    for (int64_t c = 0; c <= ncells; ++c) cell_offsets[c] = 1;
  } else {
    /* cell_offsets[c] (0-based array index c) currently holds count of cell c (1-based id c) for c>=1 */
    cell_offsets[0] = 1;
    for (int64_t c = 1; c <= ncells; ++c) cell_offsets[c] += cell_offsets[c - 1];
  }
  /* stable placement: cell c occupies [offsets[c-1], offsets[c]) (1-based) */
  int64_t* fillp = (int64_t*)malloc(sizeof(int64_t) * (ncells + 1));
  if (!fillp) {
    free(cid);
    return ORC_ERR_NOMEM;
  }
  for (int64_t c = 1; c <= ncells; ++c) fillp[c] = cell_offsets[c - 1];
  for (int64_t i = 0; i < nat; ++i) {
    int64_t pos = fillp[cid[i]]++; /* 1-based */
    perm[pos - 1] = i + 1;
  }
  for (int64_t s = 0; s < nat; ++s) {
    int64_t i = perm[s] - 1;
    cell_id_sorted[s] = cid[i];
    X_sorted[3 * s + 0] = X[3 * i + 0];
    X_sorted[3 * s + 1] = X[3 * i + 1];
    X_sorted[3 * s + 2] = X[3 * i + 2];
  }
  free(fillp);
  free(cid);
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* shared traversal, gpu_kernels.jl:58-101                             */
/* ------------------------------------------------------------------ */

typedef void (*pair_cb)(void* ctx, int64_t j, const double R[3], const int64_t S[3]);

static void winding(const orc_clist* L, const double x[3], int64_t c[3], int64_t w[3]) {
  int64_t c0[3];
  p2c(L->inv, x, L->ns, c0);
  for (int k = 0; k < 3; ++k) c[k] = wrap_and_shift(c0[k], L->ns[k], L->pbc[k], &w[k]);
}

/* R = (xj - xi) + C' * S, with S converted exactly to double */
static void pair_R(const double C[9], const double xi[3], const double xj[3], const int64_t S[3], double R[3]) {
  double Sd[3] = {(double)S[0], (double)S[1], (double)S[2]}, CS[3];
  matT_vec(C, Sd, CS);
  for (int k = 0; k < 3; ++k) R[k] = (xj[k] - xi[k]) + CS[k];
}

static void for_each_neighbour(const orc_clist* L, int64_t i /*1-based*/, pair_cb cb, void* ctx) {
  const double* xi = L->X + 3 * (i - 1);
  int64_t ci[3], wi[3];
  winding(L, xi, ci, wi);
  for (int64_t dz = -L->nxyz[2]; dz <= L->nxyz[2]; ++dz)
    for (int64_t dy = -L->nxyz[1]; dy <= L->nxyz[1]; ++dy)
      for (int64_t dx = -L->nxyz[0]; dx <= L->nxyz[0]; ++dx) {
        int64_t d[3] = {dx, dy, dz};
        /* _is_cell_in_bounds, :20-25 */
        int inb = 1;
        for (int k = 0; k < 3; ++k)
          if (!L->pbc[k] && !(1 <= ci[k] + d[k] && ci[k] + d[k] <= L->ns[k])) inb = 0;
        if (!inb) continue;
        /* _get_neighbor_cell, :39-47 */
        int64_t cj[3], sl[3];
        for (int k = 0; k < 3; ++k) cj[k] = wrap_and_shift(ci[k] + d[k], L->ns[k], L->pbc[k], &sl[k]);
        int64_t lin = sub2ind(L->ns, cj);
        int64_t a = L->cell_offsets[lin - 1], b = L->cell_offsets[lin] - 1;
        for (int64_t idx = a; idx <= b; ++idx) {
          int64_t j = L->perm[idx - 1];
          if (i == j && sl[0] == 0 && sl[1] == 0 && sl[2] == 0) continue; /* :30-33 */
          const double* xj = L->X + 3 * (j - 1);
          int64_t cjj[3], wj[3], S[3];
          winding(L, xj, cjj, wj);
          for (int k = 0; k < 3; ++k) S[k] = sl[k] + wi[k] - wj[k];
          double R[3];
          pair_R(L->C, xi, xj, S, R);
          double r2 = sa_dot(R, R);
          if (r2 < L->cutoff_sq) cb(ctx, j, R, S);
        }
      }
}

static int make_clist(orc_clist* L, const double* X, int64_t nat, const double C[9], const uint8_t pbc[3],
                      double cutoff, const int64_t* perm, const int64_t* cell_offsets) {
  L->X = X;
  L->nat = nat;
  memcpy(L->C, C, sizeof(double) * 9);
  int st = orc_analyze_cell(C, cutoff, 8, L->inv, L->ns, L->lens, L->nxyz);
  if (st) return st;
  L->ncells = L->ns[0] * L->ns[1] * L->ns[2];
  L->cutoff = cutoff;
  L->cutoff_sq = cutoff * cutoff;
  for (int k = 0; k < 3; ++k) L->pbc[k] = pbc[k] ? 1 : 0;
  L->perm = perm;
  L->cell_offsets = cell_offsets;
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* count / offsets / fill (gpu_kernels.jl:132-180, 211-219, 299-364)   */
/* threaded over atoms like the KernelAbstractions CPU backend         */
/* ------------------------------------------------------------------ */

typedef struct {
  const orc_clist* L;
  int64_t i0, i1;
  int64_t* counts;
  const int64_t* first;
  int64_t *oi, *oj, *oS;
  double* oR;
  double* per_atom;
} work_t;

static void cb_count(void* ctx, int64_t j, const double R[3], const int64_t S[3]) {
  (void)j;
  (void)R;
  (void)S;
  (*(int64_t*)ctx)++;
}

typedef struct {
  int64_t i, w;
  int64_t *oi, *oj, *oS;
  double* oR;
} fill_ctx;

static void cb_fill(void* vctx, int64_t j, const double R[3], const int64_t S[3]) {
  fill_ctx* c = (fill_ctx*)vctx;
  int64_t w = c->w++;
  c->oi[w] = c->i;
  c->oj[w] = j;
  for (int k = 0; k < 3; ++k) c->oS[3 * w + k] = S[k];
  if (c->oR)
    for (int k = 0; k < 3; ++k) c->oR[3 * w + k] = R[k];
}

typedef struct {
  double s;
} r6_ctx;

/* lazy reduction f(R) = 1 / ((r2*r2)*r2), r2 = dot(R,R), summed in traversal order */
static void cb_r6(void* vctx, int64_t j, const double R[3], const int64_t S[3]) {
  (void)j;
  (void)S;
  double r2 = sa_dot(R, R);
  ((r6_ctx*)vctx)->s += 1.0 / ((r2 * r2) * r2);
}

static void* count_worker(void* arg) {
  work_t* w = (work_t*)arg;
  for (int64_t i = w->i0; i < w->i1; ++i) {
    int64_t n = 0;
    for_each_neighbour(w->L, i + 1, cb_count, &n);
    w->counts[i] = n;
  }
  return NULL;
}

static void* fill_worker(void* arg) {
  work_t* w = (work_t*)arg;
  for (int64_t i = w->i0; i < w->i1; ++i) {
    fill_ctx c = {i + 1, w->first[i] - 1, w->oi, w->oj, w->oS, w->oR};
    for_each_neighbour(w->L, i + 1, cb_fill, &c);
  }
  return NULL;
}

static void* r6_worker(void* arg) {
  work_t* w = (work_t*)arg;
  for (int64_t i = w->i0; i < w->i1; ++i) {
    r6_ctx c = {0.0};
    for_each_neighbour(w->L, i + 1, cb_r6, &c);
    w->per_atom[i] = c.s;
  }
  return NULL;
}

static void run_threads(void* (*fn)(void*), work_t* proto, int64_t nat, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  if (nat < nthreads) nthreads = nat > 0 ? (int)nat : 1;
  pthread_t th[256];
  work_t w[256];
  for (int t = 0; t < nthreads; ++t) {
    w[t] = *proto;
    w[t].i0 = nat * t / nthreads;
    w[t].i1 = nat * (t + 1) / nthreads;
  }
  for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, fn, &w[t]);
  fn(&w[0]);
  for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
}

int orc_count(const double* X, int64_t nat, const double C[9], const uint8_t pbc[3], double cutoff,
              const int64_t* perm, const int64_t* cell_offsets, int nthreads, int64_t* counts) {
  orc_clist L;
  int st = make_clist(&L, X, nat, C, pbc, cutoff, perm, cell_offsets);
  if (st) return st;
  work_t proto = {&L, 0, 0, counts, NULL, NULL, NULL, NULL, NULL, NULL};
  run_threads(count_worker, &proto, nat, nthreads);
  return ORC_OK;
}

/* compute_pair_offsets (CPU), gpu_kernels.jl:211-219: first[1]=1, first[i+1]=first[i]+counts[i] */
void orc_pair_offsets(const int64_t* counts, int64_t nat, int64_t* first) {
  first[0] = 1;
  for (int64_t i = 0; i < nat; ++i) first[i + 1] = first[i] + counts[i];
}

int orc_fill(const double* X, int64_t nat, const double C[9], const uint8_t pbc[3], double cutoff, const int64_t* perm,
             const int64_t* cell_offsets, const int64_t* first, int nthreads, int64_t* oi, int64_t* oj, int64_t* oS,
             double* oR) {
  orc_clist L;
  int st = make_clist(&L, X, nat, C, pbc, cutoff, perm, cell_offsets);
  if (st) return st;
  work_t proto = {&L, 0, 0, NULL, first, oi, oj, oS, oR, NULL};
  run_threads(fill_worker, &proto, nat, nthreads);
  return ORC_OK;
}

int orc_lazy_r6(const double* X, int64_t nat, const double C[9], const uint8_t pbc[3], double cutoff,
                const int64_t* perm, const int64_t* cell_offsets, int nthreads, double* per_atom) {
  orc_clist L;
  int st = make_clist(&L, X, nat, C, pbc, cutoff, perm, cell_offsets);
  if (st) return st;
  work_t proto = {&L, 0, 0, NULL, NULL, NULL, NULL, NULL, NULL, per_atom};
  run_threads(r6_worker, &proto, nat, nthreads);
  return ORC_OK;
}

/* neighbours(clist, i) for one atom: returns the count; fills up to cap entries */
typedef struct {
  int64_t n, cap;
  int64_t *oj, *oS;
  double* oR;
} nb_ctx;

static void cb_nb(void* vctx, int64_t j, const double R[3], const int64_t S[3]) {
  nb_ctx* c = (nb_ctx*)vctx;
  if (c->n < c->cap) {
    c->oj[c->n] = j;
    for (int k = 0; k < 3; ++k) {
      c->oS[3 * c->n + k] = S[k];
      c->oR[3 * c->n + k] = R[k];
    }
  }
  c->n++;
}

int64_t orc_neighbours(const double* X, int64_t nat, const double C[9], const uint8_t pbc[3], double cutoff,
                       const int64_t* perm, const int64_t* cell_offsets, int64_t i, int64_t cap, int64_t* oj,
                       int64_t* oS, double* oR) {
  orc_clist L;
  if (make_clist(&L, X, nat, C, pbc, cutoff, perm, cell_offsets)) return -1;
  nb_ctx c = {0, cap, oj, oS, oR};
  for_each_neighbour(&L, i, cb_nb, &c);
  return c.n;
}

/* _getR for a list of pairs: R = (X[j] - X[i]) + C' S, cell_list.jl:525-531 */
void orc_getR(const double* X, const double C[9], int64_t np, const int64_t* oi, const int64_t* oj,
              const int64_t* oS, double* oR) {
  for (int64_t p = 0; p < np; ++p) pair_R(C, X + 3 * (oi[p] - 1), X + 3 * (oj[p] - 1), oS + 3 * p, oR + 3 * p);
}

/* ------------------------------------------------------------------ */
/* whole sort-based CPU path (build_cell_list + materialize_pairlist)  */
/* with the reference's allocation pattern; used as the timed CPU      */
/* baseline and by tests.  Outputs are malloc'd; free with orc_free.   */
/* ------------------------------------------------------------------ */

typedef struct {
  int64_t nat, npairs, ncells;
  int64_t *perm, *cell_id, *cell_offsets, *first, *i, *j, *S;
  double *X_sorted, *R;
} orc_result;

void orc_free(orc_result* r) {
  if (!r) return;
  free(r->perm);
  free(r->cell_id);
  free(r->cell_offsets);
  free(r->first);
  free(r->i);
  free(r->j);
  free(r->S);
  free(r->X_sorted);
  free(r->R);
  memset(r, 0, sizeof(*r));
}

int orc_neighbour_list(const double* X, int64_t nat, const double C[9], const uint8_t pbc[3], double cutoff,
                       int ti_bytes, int nthreads, int with_R, orc_result* out) {
  memset(out, 0, sizeof(*out));
  double inv[9], lens[3];
  int64_t ns[3], nxyz[3];
  int st = orc_analyze_cell(C, cutoff, ti_bytes, inv, ns, lens, nxyz);
  if (st) return st;
  int64_t ncells = ns[0] * ns[1] * ns[2];
  int64_t nn = nat > 0 ? nat : 1;
  out->nat = nat;
  out->ncells = ncells;
  out->perm = (int64_t*)malloc(sizeof(int64_t) * nn);
  out->cell_id = (int64_t*)malloc(sizeof(int64_t) * nn);
  out->cell_offsets = (int64_t*)malloc(sizeof(int64_t) * (ncells + 1));
  out->X_sorted = (double*)malloc(sizeof(double) * 3 * nn);
  out->first = (int64_t*)malloc(sizeof(int64_t) * (nat + 1));
  int64_t* counts = (int64_t*)malloc(sizeof(int64_t) * nn);
  if (!out->perm || !out->cell_id || !out->cell_offsets || !out->X_sorted || !out->first || !counts) {
    free(counts);
    orc_free(out);
    return ORC_ERR_NOMEM;
  }
  st = orc_build_cell_list(X, nat, C, pbc, cutoff, ti_bytes, out->perm, out->cell_id, out->cell_offsets, out->X_sorted);
  if (st) {
    free(counts);
    orc_free(out);
    return st;
  }
  st = orc_count(X, nat, C, pbc, cutoff, out->perm, out->cell_offsets, nthreads, counts);
  orc_pair_offsets(counts, nat, out->first);
  free(counts);
  int64_t np = out->first[nat] - 1;
  out->npairs = np;
  int64_t pp = np > 0 ? np : 1;
  out->i = (int64_t*)malloc(sizeof(int64_t) * pp);
  out->j = (int64_t*)malloc(sizeof(int64_t) * pp);
  out->S = (int64_t*)malloc(sizeof(int64_t) * 3 * pp);
  out->R = with_R ? (double*)malloc(sizeof(double) * 3 * pp) : NULL;
  if (!out->i || !out->j || !out->S || (with_R && !out->R)) {
    orc_free(out);
    return ORC_ERR_NOMEM;
  }
  if (np > 0)
    st = orc_fill(X, nat, C, pbc, cutoff, out->perm, out->cell_offsets, out->first, nthreads, out->i, out->j, out->S,
                  out->R);
  return st;
}

/* ------------------------------------------------------------------ */
/* legacy linked-list path, cell_list.jl:185-505                       */
/* ------------------------------------------------------------------ */

/* Julia mod(x, 1.0) for Float64: r = rem(x,y); r==0 -> copysign(r,y);
 * sign(r) != sign(y) -> r + y; else r. */
static double julia_mod1(double x) {
  double r = fmod(x, 1.0);
  if (r == 0) return copysign(r, 1.0);
  if ((r > 0) != (1.0 > 0)) return r + 1.0;
  return r;
}

/* _fix_cell_, :459-505.  X (nat x 3) and C are updated in place. */
void orc_fix_cell(double* X, int64_t nat, double C[9], const uint8_t pbc[3]) {
  double inv[9];
  sa_inv(C, inv);
  double min_lam[3] = {0, 0, 0}, max_lam[3] = {1, 1, 1};
  for (int64_t ix = 0; ix < nat; ++ix) {
    double lam[3];
    matT_vec(inv, X + 3 * ix, lam); /* inv(C)' * x */
    for (int i = 0; i < 3; ++i) {
      int update_x = 0;
      if (!(0.0 <= lam[i] && lam[i] < 1.0)) {
        if (pbc[i]) {
          lam[i] = julia_mod1(lam[i]);
          update_x = 1;
        } else {
          min_lam[i] = fmin(min_lam[i], lam[i]);
          max_lam[i] = fmax(max_lam[i], lam[i]);
        }
      }
      if (update_x) matT_vec(C, lam, X + 3 * ix); /* C' * lam */
    }
  }
  double mn = fmin(fmin(min_lam[0], min_lam[1]), min_lam[2]);
  double mx = fmax(fmax(max_lam[0], max_lam[1]), max_lam[2]);
  if (mn < 0.0 || mx > 1.0) {
    double negC[9], t[3];
    for (int k = 0; k < 9; ++k) negC[k] = -C[k];
    matT_vec(negC, min_lam, t); /* (-C') * min_lam */
    for (int64_t n = 0; n < nat; ++n)
      for (int k = 0; k < 3; ++k) X[3 * n + k] = X[3 * n + k] + t[k];
    for (int i = 0; i < 3; ++i) {
      max_lam[i] = max_lam[i] - min_lam[i];
      min_lam[i] = 0.0;
    }
    for (int i = 0; i < 3; ++i)
      if (max_lam[i] > 1) max_lam[i] = max_lam[i] * 1.01;
    /* new row k = max_lam[k] * old row k */
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) C[r + 3 * c] = max_lam[r] * C[r + 3 * c];
  }
}

typedef struct {
  int64_t n, cap;
  int64_t *i, *j, *S;
} vec_pairs;

static int push_pair(vec_pairs* v, int64_t i, int64_t j, const int64_t S[3]) {
  if (v->n == v->cap) {
    int64_t nc = v->cap ? 2 * v->cap : 1024;
    int64_t* ni = (int64_t*)realloc(v->i, sizeof(int64_t) * nc);
    if (!ni) return 1;
    v->i = ni;
    int64_t* nj = (int64_t*)realloc(v->j, sizeof(int64_t) * nc);
    if (!nj) return 1;
    v->j = nj;
    int64_t* nS = (int64_t*)realloc(v->S, sizeof(int64_t) * 3 * nc);
    if (!nS) return 1;
    v->S = nS;
    v->cap = nc;
  }
  v->i[v->n] = i;
  v->j[v->n] = j;
  for (int k = 0; k < 3; ++k) v->S[3 * v->n + k] = S[k];
  v->n++;
  return 0;
}

static int64_t bin_trunc(int64_t i, int pbc, int64_t n) { return pbc ? i : clampi(i, 1, n); }

/* truncated integer division (Julia ÷) */
static int64_t idiv_trunc(int64_t a, int64_t b) { return a / b; }

typedef struct {
  int64_t j;
  int64_t S[3];
  int64_t ord;
} jrec;

static int cmp_jrec(const void* a, const void* b) {
  const jrec* x = (const jrec*)a;
  const jrec* y = (const jrec*)b;
  if (x->j != y->j) return x->j < y->j ? -1 : 1;
  return x->ord < y->ord ? -1 : (x->ord > y->ord ? 1 : 0); /* stable */
}

/* Legacy PairList(X, cutoff, cell, pbc; fixcell).  X and C are copied
 * (the fix step may move atoms).  Returns #pairs or -status. Outputs are
 * malloc'd into out (i, j, S, first, and X_fixed/C_fixed). */
int64_t orc_legacy_pairlist(const double* X_in, int64_t nat, const double C_in[9], const uint8_t pbc_in[3],
                            double cutoff, int ti_bytes, int fixcell, orc_result* out, double C_out[9]) {
  memset(out, 0, sizeof(*out));
  uint8_t pbc[3] = {pbc_in[0] ? 1 : 0, pbc_in[1] ? 1 : 0, pbc_in[2] ? 1 : 0};
  double* X = (double*)malloc(sizeof(double) * 3 * (nat > 0 ? nat : 1));
  if (!X) return -ORC_ERR_NOMEM;
  memcpy(X, X_in, sizeof(double) * 3 * nat);
  double C[9];
  memcpy(C, C_in, sizeof(C));
  if (fixcell) orc_fix_cell(X, nat, C, pbc);
  memcpy(C_out, C, sizeof(C));
  /* _celllist_, :185-230 */
  double inv[9], lens[3];
  int64_t ns[3], nxyz[3];
  int st = orc_analyze_cell(C, cutoff, ti_bytes, inv, ns, lens, nxyz);
  if (st) {
    free(X);
    return -st;
  }
  int64_t ncells = ns[0] * ns[1] * ns[2];
  int64_t* seed = (int64_t*)malloc(sizeof(int64_t) * ncells);
  int64_t* last = (int64_t*)malloc(sizeof(int64_t) * ncells);
  int64_t* next = (int64_t*)malloc(sizeof(int64_t) * (nat > 0 ? nat : 1));
  if (!seed || !last || !next) {
    free(X);
    free(seed);
    free(last);
    free(next);
    return -ORC_ERR_NOMEM;
  }
  for (int64_t c = 0; c < ncells; ++c) seed[c] = -1;
  for (int64_t i = 1; i <= nat; ++i) {
    int64_t c[3];
    p2c(inv, X + 3 * (i - 1), ns, c);
    for (int k = 0; k < 3; ++k) c[k] = pbc[k] ? bin_wrap(c[k], ns[k]) : clampi(c[k], 1, ns[k]);
    int64_t ci = sub2ind(ns, c);
    next[i - 1] = -1;
    if (seed[ci - 1] < 0) {
      seed[ci - 1] = i;
    } else {
      next[last[ci - 1] - 1] = i;
    }
    last[ci - 1] = i;
  }
  /* _pairlist_(clist), :233-297 and _find_neighbours_!, :301-366 */
  double cutoff_sq = cutoff * cutoff;
  /* bins = hcat(C[1,:]/n1, C[2,:]/n2, C[3,:]/n3): column k = row k / n_k */
  double bins[9];
  for (int k = 0; k < 3; ++k)
    for (int r = 0; r < 3; ++r) bins[r + 3 * k] = C[k + 3 * r] / (double)ns[k];
  vec_pairs v = {0, 0, NULL, NULL, NULL};
  int oom = 0;
  for (int64_t i = 1; i <= nat && !oom; ++i) {
    const double* xi = X + 3 * (i - 1);
    int64_t ci0[3], ci[3];
    p2c(inv, xi, ns, ci0);
    for (int k = 0; k < 3; ++k) ci[k] = bin_trunc(ci0[k], pbc[k], ns[k]);
    double cim1[3] = {(double)(ci[0] - 1), (double)(ci[1] - 1), (double)(ci[2] - 1)}, bc[3], dxi[3];
    mat_vec(bins, cim1, bc);
    for (int k = 0; k < 3; ++k) dxi[k] = xi[k] - bc[k];
    for (int k = 0; k < 3; ++k) ci[k] = pbc[k] ? bin_wrap(ci0[k], ns[k]) : clampi(ci0[k], 1, ns[k]);
    for (int64_t z = -nxyz[2]; z <= nxyz[2]; ++z)
      for (int64_t y = -nxyz[1]; y <= nxyz[1]; ++y)
        for (int64_t x = -nxyz[0]; x <= nxyz[0]; ++x) {
          int64_t xyz[3] = {x, y, z}, cj[3];
          int ok = 1;
          for (int k = 0; k < 3; ++k) {
            cj[k] = pbc[k] ? bin_wrap(ci[k] + xyz[k], ns[k]) : ci[k] + xyz[k];
            if (!(1 <= cj[k] && cj[k] <= ns[k])) ok = 0;
          }
          if (!ok) continue;
          int64_t ncj = sub2ind(ns, cj);
          double xyzd[3] = {(double)x, (double)y, (double)z}, off[3];
          mat_vec(bins, xyzd, off);
          for (int64_t j = seed[ncj - 1]; j > 0; j = next[j - 1]) {
            if (!(i != j || x != 0 || y != 0 || z != 0)) continue;
            const double* xj = X + 3 * (j - 1);
            int64_t cjp[3];
            p2c(inv, xj, ns, cjp);
            for (int k = 0; k < 3; ++k) cjp[k] = bin_trunc(cjp[k], pbc[k], ns[k]);
            double cjm1[3] = {(double)(cjp[0] - 1), (double)(cjp[1] - 1), (double)(cjp[2] - 1)}, bj[3], dx[3];
            mat_vec(bins, cjm1, bj);
            for (int k = 0; k < 3; ++k) dx[k] = ((xj[k] - bj[k]) - dxi[k]) + off[k];
            double d2 = sa_dot(dx, dx);
            if (d2 < cutoff_sq) {
              int64_t S[3];
              for (int k = 0; k < 3; ++k) S[k] = idiv_trunc(ci0[k] - cjp[k] + xyz[k], ns[k]);
              if (push_pair(&v, i, j, S)) oom = 1;
            }
          }
        }
  }
  free(seed);
  free(last);
  free(next);
  if (oom) {
    free(v.i);
    free(v.j);
    free(v.S);
    free(X);
    return -ORC_ERR_NOMEM;
  }
  /* get_first, :401-418 (i ascending) */
  int64_t* first = (int64_t*)malloc(sizeof(int64_t) * (nat + 1));
  {
    int64_t idx = 1, n = 1;
    while (n <= nat && idx <= v.n) {
      first[n - 1] = idx;
      while (v.i[idx - 1] == n) {
        idx++;
        if (idx > v.n) break;
      }
      n++;
    }
    for (int64_t m = n; m <= nat + 1; ++m) first[m - 1] = v.n + 1;
  }
  /* sort_neigs!, :427-446: stable sort of each site's j, S moves along */
  int64_t maxrun = 0;
  for (int64_t n = 0; n < nat; ++n)
    if (first[n + 1] - first[n] > maxrun) maxrun = first[n + 1] - first[n];
  jrec* tmp = (jrec*)malloc(sizeof(jrec) * (maxrun > 0 ? maxrun : 1));
  for (int64_t n = 0; n < nat; ++n) {
    int64_t a = first[n] - 1, b = first[n + 1] - 1;
    if (b - a > 1) {
      for (int64_t p = a; p < b; ++p) {
        tmp[p - a].j = v.j[p];
        memcpy(tmp[p - a].S, v.S + 3 * p, sizeof(int64_t) * 3);
        tmp[p - a].ord = p;
      }
      qsort(tmp, (size_t)(b - a), sizeof(jrec), cmp_jrec);
      for (int64_t p = a; p < b; ++p) {
        v.j[p] = tmp[p - a].j;
        memcpy(v.S + 3 * p, tmp[p - a].S, sizeof(int64_t) * 3);
      }
    }
  }
  free(tmp);
  out->nat = nat;
  out->npairs = v.n;
  out->i = v.i;
  out->j = v.j;
  out->S = v.S;
  out->first = first;
  out->X_sorted = X; /* the (possibly moved) positions the legacy list refers to */
  return v.n;
}
