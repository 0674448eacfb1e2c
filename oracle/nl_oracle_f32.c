/*
 * nl_oracle_f32.c -- CPU restatement of NeighbourLists.jl (v0.6.2) with
 * positions of type T = Float32, for testing.
 *
 * TEST INFRASTRUCTURE ONLY: the correctness oracle of the GPU engine's
 * single-precision path.  Only the test suite may load it.
 *
 * The reference is generic in T: build_cell_list converts the cell and the
 * cutoff to T (src/cell_list.jl:637-639) and every floating-point operation
 * below is then a Float32 operation:
 *   - analyze_cell (inv, lengths: det, cross, norm)  src/cell_list.jl:94-95,152-170
 *   - position_to_cell_index                         src/cell_list.jl:66-74
 *   - stable sort by cell id, cell offsets           src/cell_list.jl:647-748
 *   - traversal R = xj - xi + C'S, dot < cutoff^2    src/gpu_kernels.jl:20-101
 *   - nxyz = ceil(cutoff * (ncells ./ lens))          src/gpu_kernels.jl:315-316
 *   - count / offsets / fill                         src/gpu_kernels.jl:132-237
 * with the operation order of nl_oracle.c (StaticArrays' unrolled 3x3
 * methods, left folds).  Compiled with -ffp-contract=off; C evaluates float
 * expressions in float on the supported targets (FLT_EVAL_METHOD == 0).
 * Matrices are 9 floats in column-major order; indices are 1-based int64.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define F32_OK 0
#define F32_ERR_ARG 1
#define F32_ERR_TOO_MANY_CELLS 2
#define F32_ERR_NOMEM 3

static void f_cross(const float a[3], const float b[3], float o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
static float f_dot(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
static float f_norm(const float a[3]) { return sqrtf((a[0] * a[0] + a[1] * a[1]) + a[2] * a[2]); }
static float f_det(const float M[9]) {
  float c[3];
  f_cross(M + 3, M + 6, c);
  return f_dot(M, c);
}
/* inv: the same steps as sa_inv of nl_oracle.c, in Float32 */
static void f_inv(const float M[9], float out[9]) {
  float x0[3] = {M[0], M[1], M[2]}, x1[3] = {M[3], M[4], M[5]}, x2[3] = {M[6], M[7], M[8]};
  float y0[3], y1[3], y2[3];
  f_cross(x1, x2, y0);
  float d = f_dot(x0, y0);
  for (int k = 0; k < 3; ++k) {
    x0[k] = x0[k] / d;
    y0[k] = y0[k] / d;
  }
  f_cross(x2, x0, y1);
  f_cross(x0, x1, y2);
  for (int c = 0; c < 3; ++c) {
    out[0 + 3 * c] = y0[c];
    out[1 + 3 * c] = y1[c];
    out[2 + 3 * c] = y2[c];
  }
}
static void f_row(const float M[9], int r, float v[3]) {
  v[0] = M[r];
  v[1] = M[r + 3];
  v[2] = M[r + 6];
}
/* M' * v, component k = (M[0,k] v0 + M[1,k] v1) + M[2,k] v2 */
static void f_matT_vec(const float M[9], const float v[3], float o[3]) {
  for (int k = 0; k < 3; ++k) o[k] = (M[0 + 3 * k] * v[0] + M[1 + 3 * k] * v[1]) + M[2 + 3 * k] * v[2];
}

void orc_lengths_f32(const float C[9], float lens[3]) {
  float r1[3], r2[3], r3[3], c[3];
  f_row(C, 0, r1);
  f_row(C, 1, r2);
  f_row(C, 2, r3);
  float det = f_det(C);
  f_cross(r2, r3, c);
  lens[0] = det / f_norm(c);
  f_cross(r3, r1, c);
  lens[1] = det / f_norm(c);
  f_cross(r1, r2, c);
  lens[2] = det / f_norm(c);
}

int orc_analyze_cell_f32(const float C[9], float cutoff, int ti_bytes, float inv_cell[9], int64_t ns[3], float lens[3],
                         int64_t nxyz[3]) {
  if (!(cutoff > 0)) return F32_ERR_ARG;
  f_inv(C, inv_cell);
  orc_lengths_f32(C, lens);
  /* floor(TI, x) accepts x < typemax(TI) + 1 */
  float tmax = ti_bytes == 4 ? 2147483648.0f : 9223372036854775808.0f;
  long double prod = 1;
  for (int k = 0; k < 3; ++k) {
    lens[k] = fabsf(lens[k]);
    float t = floorf(lens[k] / cutoff);
    if (!(t < tmax)) return F32_ERR_TOO_MANY_CELLS;
    ns[k] = t < 1 ? 1 : (int64_t)t;
    prod *= (long double)ns[k];
  }
  if (prod > (long double)(ti_bytes == 4 ? 2147483647.0 : 9223372036854775807.0)) return F32_ERR_TOO_MANY_CELLS;
  for (int k = 0; k < 3; ++k) nxyz[k] = (int64_t)ceilf(cutoff * ((float)ns[k] / lens[k]));
  return F32_OK;
}

/* position_to_cell_index: c = floor(frac * n + 1) with frac = inv' x */
static void f_p2c(const float inv[9], const float x[3], const int64_t ns[3], int64_t c[3]) {
  float f[3];
  f_matT_vec(inv, x, f);
  for (int k = 0; k < 3; ++k) c[k] = (int64_t)floorf(f[k] * (float)ns[k] + 1.0f);
}

static int64_t f_clampi(int64_t i, int64_t lo, int64_t hi) { return i < lo ? lo : (i > hi ? hi : i); }
static int64_t f_bin_wrap(int64_t i, int64_t n) {
  if (i <= 0) i += ((-i) / n + 1) * n;
  if (i > n) i -= ((i - 1) / n) * n;
  return i;
}
static int64_t f_wrap_and_shift(int64_t i, int64_t n, int pbc, int64_t* s) {
  if (!pbc) {
    *s = 0;
    return f_clampi(i, 1, n);
  }
  int64_t w = f_bin_wrap(i, n);
  *s = (i - w) / n;
  return w;
}
static int64_t f_sub2ind(const int64_t ns[3], const int64_t c[3]) {
  return c[0] + (c[1] - 1) * ns[0] + (c[2] - 1) * ns[0] * ns[1];
}

typedef struct {
  int64_t nat, npairs, ncells;
  int64_t *perm, *cell_id, *cell_offsets, *first, *i, *j, *S;
  float *X_sorted, *R;
} orc_result_f32;

void orc_free_f32(orc_result_f32* r) {
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

typedef struct {
  const float* X;
  float C[9], inv[9], cutoff_sq;
  int64_t ns[3], nxyz[3];
  uint8_t pbc[3];
  const int64_t *perm, *cell_offsets;
} f_clist;

/* _for_each_neighbor_pair (gpu_kernels.jl:58-101) for atom i (1-based):
 * count only (oj == NULL) or write j, S, R at w. Returns the pair count. */
static int64_t f_traverse(const f_clist* L, int64_t i, int64_t w, int64_t* oi, int64_t* oj, int64_t* oS, float* oR) {
  const float* xi = L->X + 3 * (i - 1);
  int64_t c0[3], ci[3], wi[3];
  f_p2c(L->inv, xi, L->ns, c0);
  for (int k = 0; k < 3; ++k) ci[k] = f_wrap_and_shift(c0[k], L->ns[k], L->pbc[k], &wi[k]);
  int64_t n = 0;
  for (int64_t dz = -L->nxyz[2]; dz <= L->nxyz[2]; ++dz)
    for (int64_t dy = -L->nxyz[1]; dy <= L->nxyz[1]; ++dy)
      for (int64_t dx = -L->nxyz[0]; dx <= L->nxyz[0]; ++dx) {
        int64_t d[3] = {dx, dy, dz}, cj[3], sl[3];
        int inb = 1;
        for (int k = 0; k < 3; ++k)
          if (!L->pbc[k] && !(1 <= ci[k] + d[k] && ci[k] + d[k] <= L->ns[k])) inb = 0;
        if (!inb) continue;
        for (int k = 0; k < 3; ++k) cj[k] = f_wrap_and_shift(ci[k] + d[k], L->ns[k], L->pbc[k], &sl[k]);
        int64_t lin = f_sub2ind(L->ns, cj);
        for (int64_t idx = L->cell_offsets[lin - 1]; idx < L->cell_offsets[lin]; ++idx) {
          int64_t j = L->perm[idx - 1];
          if (i == j && sl[0] == 0 && sl[1] == 0 && sl[2] == 0) continue;
          const float* xj = L->X + 3 * (j - 1);
          int64_t cj0[3], wj[3], S[3];
          f_p2c(L->inv, xj, L->ns, cj0);
          for (int k = 0; k < 3; ++k) {
            (void)f_wrap_and_shift(cj0[k], L->ns[k], L->pbc[k], &wj[k]);
            S[k] = sl[k] + wi[k] - wj[k];
          }
          float Sf[3] = {(float)S[0], (float)S[1], (float)S[2]}, CS[3], R[3];
          f_matT_vec(L->C, Sf, CS);
          for (int k = 0; k < 3; ++k) R[k] = (xj[k] - xi[k]) + CS[k];
          float r2 = f_dot(R, R);
          if (r2 < L->cutoff_sq) {
            if (oj) {
              oi[w + n] = i;
              oj[w + n] = j;
              for (int k = 0; k < 3; ++k) {
                oS[3 * (w + n) + k] = S[k];
                if (oR) oR[3 * (w + n) + k] = R[k];
              }
            }
            n++;
          }
        }
      }
  return n;
}

/* build_cell_list + materialize_pairlist with T = Float32.  X: nat x 3
 * floats; C: the cell converted to Float32 (column-major); cutoff: Float32. */
int orc_neighbour_list_f32(const float* X, int64_t nat, const float C[9], const uint8_t pbc[3], float cutoff,
                           int ti_bytes, orc_result_f32* out) {
  memset(out, 0, sizeof(*out));
  f_clist L;
  float lens[3];
  int st = orc_analyze_cell_f32(C, cutoff, ti_bytes, L.inv, L.ns, lens, L.nxyz);
  if (st) return st;
  memcpy(L.C, C, sizeof(L.C));
  L.cutoff_sq = cutoff * cutoff;
  L.X = X;
  for (int k = 0; k < 3; ++k) L.pbc[k] = pbc[k] ? 1 : 0;
  int64_t ncells = L.ns[0] * L.ns[1] * L.ns[2], nn = nat > 0 ? nat : 1;
  out->nat = nat;
  out->ncells = ncells;
  out->perm = (int64_t*)malloc(sizeof(int64_t) * nn);
  out->cell_id = (int64_t*)malloc(sizeof(int64_t) * nn);
  out->cell_offsets = (int64_t*)malloc(sizeof(int64_t) * (ncells + 1));
  out->X_sorted = (float*)malloc(sizeof(float) * 3 * nn);
  out->first = (int64_t*)malloc(sizeof(int64_t) * (nat + 1));
  int64_t* cid = (int64_t*)malloc(sizeof(int64_t) * nn);
  int64_t* fillp = (int64_t*)malloc(sizeof(int64_t) * (ncells + 1));
  if (!out->perm || !out->cell_id || !out->cell_offsets || !out->X_sorted || !out->first || !cid || !fillp) {
    free(cid);
    free(fillp);
    orc_free_f32(out);
    return F32_ERR_NOMEM;
  }
  /* _compute_cell_ids: bin_wrap_or_trunc then _sub2ind */
  for (int64_t a = 0; a < nat; ++a) {
    int64_t c[3];
    f_p2c(L.inv, X + 3 * a, L.ns, c);
    for (int k = 0; k < 3; ++k) c[k] = L.pbc[k] ? f_bin_wrap(c[k], L.ns[k]) : f_clampi(c[k], 1, L.ns[k]);
    cid[a] = f_sub2ind(L.ns, c);
  }
  /* stable sortperm by cell id and the CSR offsets (1-based) */
  for (int64_t c = 0; c <= ncells; ++c) out->cell_offsets[c] = 0;
  for (int64_t a = 0; a < nat; ++a) out->cell_offsets[cid[a]] += 1;
  out->cell_offsets[0] = 1;
  for (int64_t c = 1; c <= ncells; ++c) out->cell_offsets[c] += out->cell_offsets[c - 1];
  for (int64_t c = 1; c <= ncells; ++c) fillp[c] = out->cell_offsets[c - 1];
  for (int64_t a = 0; a < nat; ++a) out->perm[fillp[cid[a]]++ - 1] = a + 1;
  for (int64_t s = 0; s < nat; ++s) {
    int64_t a = out->perm[s] - 1;
    out->cell_id[s] = cid[a];
    for (int k = 0; k < 3; ++k) out->X_sorted[3 * s + k] = X[3 * a + k];
  }
  free(cid);
  free(fillp);
  L.perm = out->perm;
  L.cell_offsets = out->cell_offsets;
  /* count, pair offsets, fill */
  out->first[0] = 1;
  for (int64_t a = 0; a < nat; ++a) out->first[a + 1] = out->first[a] + f_traverse(&L, a + 1, 0, NULL, NULL, NULL, NULL);
  int64_t np = out->first[nat] - 1, pp = np > 0 ? np : 1;
  out->npairs = np;
  out->i = (int64_t*)malloc(sizeof(int64_t) * pp);
  out->j = (int64_t*)malloc(sizeof(int64_t) * pp);
  out->S = (int64_t*)malloc(sizeof(int64_t) * 3 * pp);
  out->R = (float*)malloc(sizeof(float) * 3 * pp);
  if (!out->i || !out->j || !out->S || !out->R) {
    orc_free_f32(out);
    return F32_ERR_NOMEM;
  }
  for (int64_t a = 0; a < nat; ++a) f_traverse(&L, a + 1, out->first[a] - 1, out->i, out->j, out->S, out->R);
  return F32_OK;
}
