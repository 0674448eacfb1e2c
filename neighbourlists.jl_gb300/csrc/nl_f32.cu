// Single-precision path: the reference with T = Float32.
//
//   position_to_cell_index (cell_list.jl:66-74)     bin32 / k_bin32 / k_prepare32
//   _for_each_neighbor_pair (gpu_kernels.jl:58-101) k_pairs32 (count and fill)
//
// The sort (scan, scatter, stable fix-up) is the double-precision path's
// (nl_build.cu, instantiated for float positions).  Every floating-point
// operation is an explicit round-to-nearest FP32 intrinsic, so nvcc cannot
// contract a product and a sum into one FMA: the reference rounds each
// operation separately.  No screen band is needed: the distance test itself
// is the reference's FP32 arithmetic, and FP32 is the fast pipe.
#include "nl_f32.cuh"
#include "nl_pairs.cuh"

namespace nl {

namespace {

inline int grid_for(long long n, int block, int max_blocks) {
  long long g = (n + block - 1) / block;
  if (g > max_blocks) g = max_blocks;
  return g < 1 ? 1 : int(g);
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// frac_k = (inv' x)_k, StaticArrays order (a1*b1 + a2*b2) + a3*b3
__device__ __forceinline__ float frac32(const float* inv, float x0, float x1, float x2, int k) {
  return fadd(fadd(fmul(inv[3 * k + 0], x0), fmul(inv[3 * k + 1], x1)), fmul(inv[3 * k + 2], x2));
}

// (C' S)_k with S converted to Float32, as the reference promotes Int * Float32
__device__ __forceinline__ float cts32(const float* C, int s0, int s1, int s2, int k) {
  return fadd(fadd(fmul(C[3 * k + 0], float(s0)), fmul(C[3 * k + 1], float(s1))), fmul(C[3 * k + 2], float(s2)));
}

// c0 = floor(frac * n + 1) in Float32, then wrap / clamp with the winding.
// false: a position that cannot be binned (non-finite, |frac * n| >= 2^30,
// or a winding beyond the record's 10-bit field).
__device__ __forceinline__ bool bin32(const Geo32& g, float x0, float x1, float x2, int c[3], int w[3]) {
  bool ok = isfinite(x0) && isfinite(x1) && isfinite(x2);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float y = fmul(frac32(g.inv, x0, x1, x2, k), float(g.ns[k]));
    float yp = fadd(y, 1.0f);
    if (!(fabsf(yp) < 1073741824.0f)) {
      ok = false;
      yp = 1.0f;
    }
    int s;
    c[k] = wrap_shift(int(floorf(yp)), g.ns[k], g.pbc[k], s);
    if (s < -(kW32Bias - 1) || s > kW32Bias - 1) {
      ok = false;
      s = 0;
    }
    w[k] = s;
  }
  return ok;
}

__device__ __forceinline__ float4 record32(float x0, float x1, float x2, const int w[3]) {
  return make_float4(x0, x1, x2, __uint_as_float(pack10(w[0] + kW32Bias, w[1] + kW32Bias, w[2] + kW32Bias)));
}

// One thread per atom (original order): cell id, ticket, record, histogram
// (the same outputs as the double-precision binning).  Batches: the atom's
// system by a binary search over the atom offsets, its geometry from the
// table, its cell index offset by the system's first cell.
template <bool BATCH>
__global__ void __launch_bounds__(256) k_bin32(Geo32 g1, const Geo32* __restrict__ geos, const int* __restrict__ atom0,
                                               const int* __restrict__ cell0, int nsys, const float* __restrict__ X,
                                               int nat, int* __restrict__ cid, int* __restrict__ ticket,
                                               float4* __restrict__ rec, int* __restrict__ cell_count,
                                               unsigned* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < nat; base += stride) {
    const long long i = base + lane;
    const bool valid = i < nat;
    int c = 0;
    if (valid) {
      const int sys = BATCH ? batch_system(atom0, nsys, int(i)) : 0;
      const Geo32& g = BATCH ? geos[sys] : g1;
      const float x0 = X[3 * i + 0], x1 = X[3 * i + 1], x2 = X[3 * i + 2];
      int cc[3], w[3];
      if (!bin32(g, x0, x1, x2, cc, w)) atomicOr(err, kFlagBadPosition);
      c = (cc[0] - 1) + g.ns[0] * ((cc[1] - 1) + g.ns[1] * (cc[2] - 1)) + (BATCH ? cell0[sys] : 0);
      rec[i] = record32(x0, x1, x2, w);
      cid[i] = c;
    }
    const int key = valid ? c : -1 - lane;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    int b = 0;
    if (valid && lane == leader) b = atomicAdd(&cell_count[c], __popc(peers));
    b = __shfl_sync(0xffffffffu, b, leader);
    if (valid) ticket[i] = b + __popc(peers & lanemask_lt());
  }
}

template <typename TI>
__global__ void __launch_bounds__(256) k_prepare32(Geo32 g, const float* __restrict__ Xs,
                                                   const TI* __restrict__ cell_id, const TI* __restrict__ perm, int nat,
                                                   float4* __restrict__ rec_sorted, int* __restrict__ scell,
                                                   unsigned* __restrict__ err) {
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < nat; s += (long long)gridDim.x * blockDim.x) {
    const float x0 = Xs[3 * s + 0], x1 = Xs[3 * s + 1], x2 = Xs[3 * s + 2];
    int cc[3], w[3];
    if (!bin32(g, x0, x1, x2, cc, w)) atomicOr(err, kFlagBadPosition);
    rec_sorted[s] = record32(x0, x1, x2, w);
    const int c = (cc[0] - 1) + g.ns[0] * ((cc[1] - 1) + g.ns[1] * (cc[2] - 1));
    scell[s] = c;
    if ((long long)cell_id[s] != (long long)c + 1) atomicOr(err, kFlagInconsistent);
    if ((long long)perm[s] < 1 || (long long)perm[s] > nat) atomicOr(err, kFlagInconsistent);
  }
}

constexpr int kW32Warps = 4;    // warps per block of the pair kernel
// candidates held per lane (a tile is 32 times that) and resident blocks per
// SM the register budget is sized for, for the count and the fill kernels
#ifndef NL_F32_PER_COUNT
#define NL_F32_PER_COUNT 2
#endif
#ifndef NL_F32_MIN_COUNT
#define NL_F32_MIN_COUNT 8
#endif
#ifndef NL_F32_PER_FILL
#define NL_F32_PER_FILL 4
#endif
#ifndef NL_F32_MIN_FILL
#define NL_F32_MIN_FILL 4
#endif

// A staged candidate's tag: s_loop + 128 in three 8-bit fields, bit 24 =
// (s_loop == 0), bit 25 = (the candidate has a winding), bit 26 = valid.
constexpr unsigned kTagLoopZero = 1u << 24;
constexpr unsigned kTagWound = 1u << 25;
constexpr unsigned kTagValid = 1u << 26;

struct Shared32 {
  float hx[32], hy[32], hz[32];  // home atoms of the group
  int hw[32][3];                 // their windings
  int hid[32];                   // their 1-based original indices
  int incl[32];                  // stencil chunk: inclusive candidate counts
  int start[32];                 // first sorted slot of the cell
  unsigned loop[32];             // s_loop + 128 packed in 8-bit fields
  float lc[3][32];               // C' s_loop
};

__device__ __forceinline__ int tag_s(unsigned t, int k) { return int((t >> (8 * k)) & 255u) - 128; }

// One warp per home cell.  The candidates of the cell's stencil -- cells in
// the reference's order dz, dy, dx (dx fastest), each cell's atoms in sorted
// order -- are taken a tile at a time into registers (kW32Per per lane,
// candidate r*32 + lane); every home atom of the cell (groups of 32, read by
// broadcast from shared memory) is tested against them in that order:
// S = s_loop + wi - wj, R = (xj - xi) + C'S, dot(R, R) < cutoff^2, all in
// FP32 with the reference's operation order, skipping i itself at zero cell
// shift (gpu_kernels.jl:58-101).  Count: pairs per atom.  Fill: accepted
// pairs are ballot-compacted to consecutive positions from first[i], so each
// atom's pairs are in the reference's traversal order.  Batches: the warp
// takes the system of its home cell from the per-cell table, copies the
// system's geometry to shared memory when the system changes, and adds the
// system's first slot to its (system-local) cell offsets and atom indices.
template <typename TI, bool FILL, bool BATCH>
__global__ void __launch_bounds__(kW32Warps * 32, FILL ? NL_F32_MIN_FILL : NL_F32_MIN_COUNT)
    k_pairs32(Pairs32Args<TI> a) {
  // count: the symmetric pass counted; fill: the count recorded in the
  // workspace that the mask write pass takes over (sym_fail == 0)
  if ((FILL || a.sym) && *a.sym_fail == 0) return;
  constexpr int kW32Per = FILL ? NL_F32_PER_FILL : NL_F32_PER_COUNT;
  constexpr int kW32Tile = 32 * kW32Per;
  __shared__ Shared32 sh_all[kW32Warps];
  __shared__ Geo32 geo_w[BATCH ? kW32Warps : 1];
  const int lane = threadIdx.x & 31;
  Shared32& W = sh_all[threadIdx.x >> 5];
  const Geo32& g = BATCH ? geo_w[threadIdx.x >> 5] : a.g;
  const unsigned lt = lanemask_lt();
  int wx = 2 * g.nxyz[0] + 1, wy = 2 * g.nxyz[1] + 1;
  int nst = wx * wy * (2 * g.nxyz[2] + 1);
  const int nwarps = gridDim.x * kW32Warps;
  const int ncells = BATCH ? a.ncells_total : g.ncells;
  int cur_sys = -1, abase = 0, coff = 0;

  // batches: the next cell (second launch: the next listed round) from a
  // counter as warps free up (uneven cells)
  const bool split = BATCH && a.rounds;
  const bool rpass = split && a.round_pass;
  const int rcap = a.nat_total / 32 + 2;  // rounds the list holds
  const int niter = rpass ? min(*a.n_rounds, rcap) : ncells;
  int* ctr = rpass ? a.round_work + (FILL ? 1 : 0) : a.work + (FILL ? 1 : 0);
  auto next_cell = [&](int cur) -> int {
    if (!BATCH) return cur + nwarps;
    int b = 0;
    if (lane == 0) b = atomicAdd(ctr, 1);
    return __shfl_sync(0xffffffffu, b, 0);
  };
  for (int idx = BATCH ? next_cell(0) : blockIdx.x * kW32Warps + (threadIdx.x >> 5); idx < niter;
       idx = next_cell(idx)) {
    const int cell = rpass ? max(min(a.rounds[idx].x, ncells - 1), 0) : idx;
    int hl = cell;  // the cell within its system
    if constexpr (BATCH) {
      const int sys = max(min(a.cell_sys[cell], a.nsys - 1), 0);
      if (sys != cur_sys) {  // the system's geometry to shared memory
        __syncwarp();
        const int* src = reinterpret_cast<const int*>(a.geos + sys);
        int* dst = reinterpret_cast<int*>(&geo_w[threadIdx.x >> 5]);
        for (int k = lane; k < int(sizeof(Geo32) / 4); k += 32) dst[k] = src[k];
        __syncwarp();
        wx = 2 * g.nxyz[0] + 1;
        wy = 2 * g.nxyz[1] + 1;
        nst = wx * wy * (2 * g.nxyz[2] + 1);
        cur_sys = sys;
      }
      abase = a.sys_atom[sys];
      coff = a.sys_cell[sys] + sys;  // the system's cell_offsets: ncells_s + 1 entries
      hl = cell - a.sys_cell[sys];
    }
    const int hs = int(a.cell_offsets[coff + hl]) - 1 + abase, he = int(a.cell_offsets[coff + hl + 1]) - 1 + abase;
    if (hs >= he) continue;
    const int ci[3] = {hl % g.ns[0] + 1, (hl / g.ns[0]) % g.ns[1] + 1, hl / (g.ns[0] * g.ns[1]) + 1};
    int hb0 = hs, hb1 = he;  // the home atoms this warp takes
    if (rpass) {
      hb0 = min(hs + 32 * max(a.rounds[idx].y, 0), he);
      hb1 = min(hb0 + 32, he);
    } else if (split && he - hs > 32) {
      hb1 = hs + 32;
      if constexpr (!FILL) {  // the count pass lists the other rounds (the fill pass reads the same list)
        const int nr = ((he - hs + 31) >> 5) - 1;
        int base = 0;
        if (lane == 0) base = atomicAdd(a.n_rounds, nr);
        base = __shfl_sync(0xffffffffu, base, 0);
        for (int k = lane; k < nr; k += 32)
          if (base + k < rcap) a.rounds[base + k] = make_int2(cell, k + 1);
      }
    }
    for (int h0 = hb0; h0 < hb1; h0 += 32) {
      const int nh = min(32, he - h0);
      // this lane's home atom: running count (fill: write offset) and range
      int hcount = 0, hn = 0;
      long long hbase = 0;
      bool hok = false;
      __syncwarp();
      if (lane < nh) {
        const float4 rh = a.rec[h0 + lane];
        const unsigned mh = __float_as_uint(rh.w);
        const int id = int(a.perm[h0 + lane]);
        W.hx[lane] = rh.x;
        W.hy[lane] = rh.y;
        W.hz[lane] = rh.z;
        W.hw[lane][0] = field10(mh, 0) - kW32Bias;
        W.hw[lane][1] = field10(mh, 1) - kW32Bias;
        W.hw[lane][2] = field10(mh, 2) - kW32Bias;
        W.hid[lane] = id;
        if constexpr (FILL) {
          hbase = (long long)a.first[abase + id - 1] - 1;
          hn = int((long long)a.first[abase + id] - 1 - hbase);
          hok = hbase >= 0 && hn >= 0 && hbase + hn <= a.capacity;
          if (!hok) atomicOr(a.err, kFlagCapacity);
        }
      }
      __syncwarp();
      for (int q0 = 0; q0 < nst; q0 += 32) {
        // stencil chunk: one cell per lane
        const int q = q0 + lane;
        bool valid = q < nst;
        const int d[3] = {q % wx - g.nxyz[0], (q / wx) % wy - g.nxyz[1], q / (wx * wy) - g.nxyz[2]};
        int cj[3], sl[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          if (!g.pbc[k] && (ci[k] + d[k] < 1 || ci[k] + d[k] > g.ns[k])) valid = false;
          cj[k] = wrap_shift(ci[k] + d[k], g.ns[k], g.pbc[k], sl[k]);
        }
        int st = 0, cnt = 0;
        if (valid) {
          const int lin = (cj[0] - 1) + g.ns[0] * ((cj[1] - 1) + g.ns[1] * (cj[2] - 1));
          st = int(a.cell_offsets[coff + lin]) - 1 + abase;
          cnt = int(a.cell_offsets[coff + lin + 1]) - 1 + abase - st;
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        if (total == 0) continue;
        __syncwarp();
        W.incl[lane] = incl;
        W.start[lane] = st;
        W.loop[lane] = (unsigned(sl[0] + 128) & 255u) | ((unsigned(sl[1] + 128) & 255u) << 8) |
                       ((unsigned(sl[2] + 128) & 255u) << 16);
        W.lc[0][lane] = valid ? cts32(g.C, sl[0], sl[1], sl[2], 0) : 0.f;
        W.lc[1][lane] = valid ? cts32(g.C, sl[0], sl[1], sl[2], 1) : 0.f;
        W.lc[2][lane] = valid ? cts32(g.C, sl[0], sl[1], sl[2], 2) : 0.f;
        __syncwarp();
        for (int t0 = 0; t0 < total; t0 += kW32Tile) {
          // this lane's candidates t0 + r*32 + lane, in registers
          float cxr[kW32Per], cyr[kW32Per], czr[kW32Per], ex[kW32Per], ey[kW32Per], ez[kW32Per];
          unsigned tag[kW32Per];
          int jor[kW32Per], jslot[kW32Per];
#pragma unroll
          for (int r = 0; r < kW32Per; ++r) {
            const int p = t0 + r * 32 + lane;
            tag[r] = 0u;
            cxr[r] = cyr[r] = czr[r] = ex[r] = ey[r] = ez[r] = 0.f;
            jor[r] = jslot[r] = 0;
            if (p < total) {
              int lo = 0, hi = 31;  // first stencil lane whose inclusive count exceeds p
              while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (W.incl[mid] > p)
                  hi = mid;
                else
                  lo = mid + 1;
              }
              const int js = W.start[lo] + (p - (lo ? W.incl[lo - 1] : 0));
              const float4 rj = a.rec[js];
              const unsigned lp = W.loop[lo];
              const bool wound = (__float_as_uint(rj.w) & kMetaFields) != pack10(kW32Bias, kW32Bias, kW32Bias);
              cxr[r] = rj.x;
              cyr[r] = rj.y;
              czr[r] = rj.z;
              ex[r] = W.lc[0][lo];
              ey[r] = W.lc[1][lo];
              ez[r] = W.lc[2][lo];
              jor[r] = int(a.perm[js]);
              jslot[r] = js;
              tag[r] = lp | (lp == 0x808080u ? kTagLoopZero : 0u) | (wound ? kTagWound : 0u) | kTagValid;
            }
          }
          for (int h = 0; h < nh; ++h) {
            const float xi = W.hx[h], yi = W.hy[h], zi = W.hz[h];
            const int wi0 = W.hw[h][0], wi1 = W.hw[h][1], wi2 = W.hw[h][2];
            const int iid = W.hid[h];
            const bool hwound = (wi0 | wi1 | wi2) != 0;
            int off = 0, nmax = 0;
            long long base = 0;
            bool ok = false;
            if constexpr (FILL) {
              off = __shfl_sync(0xffffffffu, hcount, h);
              nmax = __shfl_sync(0xffffffffu, hn, h);
              base = __shfl_sync(0xffffffffu, hbase, h);
              ok = __shfl_sync(0xffffffffu, hok ? 1 : 0, h) != 0;
            }
            int added = 0;
#pragma unroll
            for (int r = 0; r < kW32Per; ++r) {
              if (t0 + r * 32 >= total) break;  // warp-uniform
              const unsigned tg = tag[r];
              bool acc = false;
              float R0 = 0.f, R1 = 0.f, R2 = 0.f;
              int S0 = tag_s(tg, 0), S1 = tag_s(tg, 1), S2 = tag_s(tg, 2);
              if ((tg & kTagValid) && !((tg & kTagLoopZero) && jor[r] == iid)) {
                float e0 = ex[r], e1 = ey[r], e2 = ez[r];
                if (hwound || (tg & kTagWound)) {  // S = s_loop + wi - wj, C'S again
                  const unsigned mj = __float_as_uint(a.rec[jslot[r]].w);
                  S0 += wi0 - (field10(mj, 0) - kW32Bias);
                  S1 += wi1 - (field10(mj, 1) - kW32Bias);
                  S2 += wi2 - (field10(mj, 2) - kW32Bias);
                  e0 = cts32(g.C, S0, S1, S2, 0);
                  e1 = cts32(g.C, S0, S1, S2, 1);
                  e2 = cts32(g.C, S0, S1, S2, 2);
                }
                R0 = fadd(fsub(cxr[r], xi), e0);
                R1 = fadd(fsub(cyr[r], yi), e1);
                R2 = fadd(fsub(czr[r], zi), e2);
                const float r2 = fadd(fadd(fmul(R0, R0), fmul(R1, R1)), fmul(R2, R2));
                acc = r2 < g.cutoff_sq;
                if (a.half && acc)  // half list: j > i, or the atom's own image with S > 0 lexicographically
                  acc = jor[r] != iid ? jor[r] > iid : (S0 > 0 || (S0 == 0 && (S1 > 0 || (S1 == 0 && S2 > 0))));
              }
              const unsigned mask = __ballot_sync(0xffffffffu, acc);
              if constexpr (FILL) {
                const int k = off + added + __popc(mask & lt);
                if (acc && ok && k < nmax) {
                  const long long pos = base + k;
                  a.oi[pos] = TI(iid);
                  a.oj[pos] = TI(jor[r]);
                  a.oS[3 * pos + 0] = TI(S0);
                  a.oS[3 * pos + 1] = TI(S1);
                  a.oS[3 * pos + 2] = TI(S2);
                  if (a.oR) {
                    a.oR[3 * pos + 0] = R0;
                    a.oR[3 * pos + 1] = R1;
                    a.oR[3 * pos + 2] = R2;
                  }
                }
              }
              added += __popc(mask);
            }
            if (lane == h) hcount += added;
          }
        }
      }
      if (lane < nh) {
        if constexpr (FILL) {
          if (hok && hcount != hn) atomicOr(a.err, kFlagInconsistent);
        } else {
          a.counts[abase + W.hid[lane] - 1] = hcount;
        }
      }
    }
  }
}

// ------------------------------------------------------------------------
// Symmetric count pass in Float32 (27-cell stencils of distinct cells).  The
// reference's FP32 decision for (i, j, S) and (j, i, -S) is the same:
// R(j, i, -S) = -R(i, j, S) bit for bit under round-to-nearest.  As in the
// Float64 engine, the warp of home cell A tests its atoms against the
// centre and the 13 stencil cells after it, with the exact FP32 test, and
// stores every atom's accepted neighbours as one 32-bit mask per stencil
// cell (27 words per atom: rows for A's atoms, mirrored columns for the
// candidates; words whose mirrored cell is empty or outside an open axis are
// written as 0 by the atom's own warp), counts with atomics, and the cell's
// stencil table (first slot and loop shift of each stencil cell) for the
// write pass.  A cell of more than 32 atoms sets sym_fail: the per-cell
// passes run instead.
constexpr int kSym32Warps = 4;
constexpr int kSym32Chunk = 128;

struct Sym32Smem {
  float cx[kSym32Chunk], cy[kSym32Chunk], cz[kSym32Chunk];  // candidate coordinates
  float ex[kSym32Chunk], ey[kSym32Chunk], ez[kSym32Chunk];  // C' s_loop of its stencil cell
  unsigned ctag[kSym32Chunk];  // s_loop + 128 in 8-bit fields | q << 24 (bits 24-28) | wound << 29
  int cjor[kSym32Chunk];       // 1-based original index
  int cslot[kSym32Chunk];      // sorted slot
  unsigned char cbit[kSym32Chunk];  // index of the candidate in its cell
  unsigned ccol[kSym32Chunk];  // home atoms that accepted the candidate
  unsigned rmask[32][15];      // rows of the home atoms, q = 13..26
  float hx[32], hy[32], hz[32];
  int hw[32][3];
  int hid[32];                 // 1-based original index
};

__device__ __forceinline__ unsigned* sym32_table(unsigned* masks, int nat, int cell) {
  return masks + 27LL * nat + 54LL * cell;
}

template <typename TI>
__global__ void __launch_bounds__(kSym32Warps * 32, 8) k_pairs32_sym(Pairs32Args<TI> a) {
  __shared__ Sym32Smem sm_all[kSym32Warps];
  const int lane = threadIdx.x & 31;
  Sym32Smem& W = sm_all[threadIdx.x >> 5];
  const Geo32& g = a.g;
  const unsigned lt = lanemask_lt();
  const unsigned wzero = pack10(kW32Bias, kW32Bias, kW32Bias);
  for (int h = blockIdx.x * kSym32Warps + (threadIdx.x >> 5); h < g.ncells; h += gridDim.x * kSym32Warps) {
    const int hs = int(a.cell_offsets[h]) - 1, he = int(a.cell_offsets[h + 1]) - 1;
    const int nb = he - hs;
    if (nb <= 0) continue;
    const int ci[3] = {h % g.ns[0] + 1, (h / g.ns[0]) % g.ns[1] + 1, h / (g.ns[0] * g.ns[1]) + 1};
    // stencil cell q = lane (dx fastest, then dy, dz)
    int cstart = 0, ccount = 0, sl[3] = {0, 0, 0};
    bool valid = lane < 27;
    if (valid) {
      const int d[3] = {lane % 3 - 1, (lane / 3) % 3 - 1, lane / 9 - 1};
      int cj[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (!g.pbc[k] && (ci[k] + d[k] < 1 || ci[k] + d[k] > g.ns[k])) valid = false;
        cj[k] = wrap_shift(ci[k] + d[k], g.ns[k], g.pbc[k], sl[k]);
      }
      if (valid) {
        const int lin = (cj[0] - 1) + g.ns[0] * ((cj[1] - 1) + g.ns[1] * (cj[2] - 1));
        cstart = int(a.cell_offsets[lin]) - 1;
        ccount = int(a.cell_offsets[lin + 1]) - 1 - cstart;
      }
    }
    if (nb > 32 || __any_sync(0xffffffffu, ccount > 32)) {
      if (lane == 0) atomicOr(a.sym_fail, 1);
      continue;
    }
    const unsigned slp = (unsigned(sl[0] + 128) & 255u) | ((unsigned(sl[1] + 128) & 255u) << 8) |
                         ((unsigned(sl[2] + 128) & 255u) << 16);
    const float lc0 = cts32(g.C, sl[0], sl[1], sl[2], 0), lc1 = cts32(g.C, sl[0], sl[1], sl[2], 1),
                lc2 = cts32(g.C, sl[0], sl[1], sl[2], 2);
    if (lane < 27) {
      unsigned* tab = sym32_table(a.masks, g.nat, h);
      tab[lane] = unsigned(cstart);
      tab[27 + lane] = slp;
    }
    // words of the home atoms that no other warp writes
    const unsigned zq = __ballot_sync(0xffffffffu, lane < 13 && (!valid || ccount == 0));
    if (zq)
      for (int t = lane; t < nb * 13; t += 32) {
        const int at = t / 13, q = t - 13 * at;
        if ((zq >> q) & 1u) a.masks[27LL * (hs + at) + q] = 0u;
      }
    __syncwarp();
    if (lane < nb) {
      const float4 r = a.rec[hs + lane];
      const unsigned m = __float_as_uint(r.w);
      W.hx[lane] = r.x;
      W.hy[lane] = r.y;
      W.hz[lane] = r.z;
      W.hw[lane][0] = field10(m, 0) - kW32Bias;
      W.hw[lane][1] = field10(m, 1) - kW32Bias;
      W.hw[lane][2] = field10(m, 2) - kW32Bias;
      W.hid[lane] = int(a.perm[hs + lane]);
    }
#pragma unroll
    for (int k = 0; k < 14; ++k) W.rmask[lane][k] = 0u;
    // candidates: the centre and the cells after it (lanes 13..26), flattened
    const int scnt = lane >= 13 ? ccount : 0;
    int incl = scnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    const int tg = __shfl_sync(0xffffffffu, incl, 31);
    __syncwarp();
    for (int cb = 0; cb < tg; cb += kSym32Chunk) {
      const int nch = min(kSym32Chunk, tg - cb);
      for (int f0 = 0; f0 < nch; f0 += 32) {
        const int f = f0 + lane;
        const int gf = cb + min(f, nch - 1);
        int q = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
          const int v = __shfl_sync(0xffffffffu, incl, q + step - 1);
          if (v <= gf) q += step;
        }
        const int q_incl = __shfl_sync(0xffffffffu, incl, q);
        const int q_cnt = __shfl_sync(0xffffffffu, scnt, q);
        const int q_start = __shfl_sync(0xffffffffu, cstart, q);
        const unsigned q_slp = __shfl_sync(0xffffffffu, slp, q);
        const float q0 = __shfl_sync(0xffffffffu, lc0, q), q1 = __shfl_sync(0xffffffffu, lc1, q),
                    q2 = __shfl_sync(0xffffffffu, lc2, q);
        if (f < nch) {
          const int bit = gf - (q_incl - q_cnt);
          const int js = q_start + bit;
          const float4 r = a.rec[js];
          const bool wound = (__float_as_uint(r.w) & kMetaFields) != wzero;
          W.cx[f] = r.x;
          W.cy[f] = r.y;
          W.cz[f] = r.z;
          W.ex[f] = q0;
          W.ey[f] = q1;
          W.ez[f] = q2;
          W.ctag[f] = (q_slp & 0xFFFFFFu) | (unsigned(q) << 24) | (wound ? (1u << 29) : 0u);
          W.cjor[f] = int(a.perm[js]);
          W.cslot[f] = js;
          W.cbit[f] = (unsigned char)bit;
          W.ccol[f] = 0u;
        }
      }
      __syncwarp();
      for (int at = 0; at < nb; ++at) {
        const float xi = W.hx[at], yi = W.hy[at], zi = W.hz[at];
        const int wi0 = W.hw[at][0], wi1 = W.hw[at][1], wi2 = W.hw[at][2];
        const int iid = W.hid[at];
        const bool hwound = (wi0 | wi1 | wi2) != 0;
        for (int c0 = 0; c0 < nch; c0 += 32) {
          const int f = c0 + lane;
          bool acc = false;
          unsigned tg2 = 0;
          if (f < nch) {
            tg2 = W.ctag[f];
            const int q = int((tg2 >> 24) & 31u);
            if (!(q == 13 && W.cjor[f] == iid)) {  // i itself at zero loop shift (the centre)
              float e0 = W.ex[f], e1 = W.ey[f], e2 = W.ez[f];
              if (hwound || (tg2 & (1u << 29))) {
                const unsigned mj = __float_as_uint(a.rec[W.cslot[f]].w);
                const int S0 = tag_s(tg2, 0) + wi0 - (field10(mj, 0) - kW32Bias);
                const int S1 = tag_s(tg2, 1) + wi1 - (field10(mj, 1) - kW32Bias);
                const int S2 = tag_s(tg2, 2) + wi2 - (field10(mj, 2) - kW32Bias);
                e0 = cts32(g.C, S0, S1, S2, 0);
                e1 = cts32(g.C, S0, S1, S2, 1);
                e2 = cts32(g.C, S0, S1, S2, 2);
              }
              const float R0 = fadd(fsub(W.cx[f], xi), e0);
              const float R1 = fadd(fsub(W.cy[f], yi), e1);
              const float R2 = fadd(fsub(W.cz[f], zi), e2);
              acc = fadd(fadd(fmul(R0, R0), fmul(R1, R1)), fmul(R2, R2)) < g.cutoff_sq;
            }
          }
          if (acc) {
            const int q = int((tg2 >> 24) & 31u);
            atomicOr(&W.rmask[at][q - 13], 1u << W.cbit[f]);
            if (q > 13) W.ccol[f] |= 1u << at;
          }
        }
      }
      __syncwarp();
      for (int f = lane; f < nch; f += 32) {
        const int q = int((W.ctag[f] >> 24) & 31u);
        if (q > 13) {
          const unsigned cc = W.ccol[f];
          a.masks[27LL * W.cslot[f] + (26 - q)] = cc;
          if (cc) atomicAdd(a.counts + (W.cjor[f] - 1), __popc(cc));
        }
      }
      __syncwarp();
    }
    for (int t = lane; t < nb * 14; t += 32) {
      const int at = t / 14, k = t - 14 * at;
      a.masks[27LL * (hs + at) + 13 + k] = W.rmask[at][k];
    }
    if (lane < nb) {
      int c = 0;
#pragma unroll
      for (int k = 0; k < 14; ++k) c += __popc(W.rmask[lane][k]);
      if (c) atomicAdd(a.counts + (W.hid[lane] - 1), c);
    }
    __syncwarp();
  }
}

// k-th (0-based) set bit of m (m has more than k set bits)
__device__ __forceinline__ int kth_bit32(unsigned m, int k) {
  int pos = 0;
#pragma unroll
  for (int w = 16; w > 0; w >>= 1) {
    const int c = __popc(m & ((1u << w) - 1u));
    if (c <= k) {
      k -= c;
      m >>= w;
      pos += w;
    }
  }
  return pos;
}

// Write pass from the masks: one warp per atom at a time.  Lane q holds the
// atom's mask word q; lane r of a pass takes the atom's r-th pair (stencil
// cell by a shuffle search over the prefix counts, atom by a popcount
// select), gathers it and writes i, j, S, R (FP32, the reference's
// arithmetic) at first[i] + r.
template <typename TI>
__global__ void __launch_bounds__(128) k_emit32_masks(Pairs32Args<TI> a) {
  if (*a.sym_fail) return;
  const Geo32& g = a.g;
  const int lane = threadIdx.x & 31;
  const unsigned lt = lanemask_lt();
  const int stride = gridDim.x * 4;
  // the next atom's own loads (record, index, mask word, cell) are issued
  // before this atom's pairs, so their latency overlaps its work
  int s = blockIdx.x * 4 + (threadIdx.x >> 5);
  float4 nx_ri = make_float4(0.f, 0.f, 0.f, 0.f);
  TI nx_iid = 1;
  unsigned nx_m = 0u;
  int nx_cell = 0;
  auto fetch = [&](int t) {
    if (t < g.nat) {
      nx_ri = a.rec[t];
      nx_iid = a.perm[t];
      nx_m = lane < 27 ? a.masks[27LL * t + lane] : 0u;
      nx_cell = a.scell[t];
    }
  };
  fetch(s);
  for (; s < g.nat; s += stride) {
    const float4 ri = nx_ri;
    const TI iid = nx_iid;
    const unsigned m = nx_m;
    const int cell = nx_cell;
    fetch(s + stride);
    const unsigned mi = __float_as_uint(ri.w);
    const int wi0 = field10(mi, 0) - kW32Bias, wi1 = field10(mi, 1) - kW32Bias, wi2 = field10(mi, 2) - kW32Bias;
    const long long base = (long long)a.first[iid - 1] - 1;
    const long long nexp = (long long)a.first[iid] - 1 - base;
    const unsigned* tab = sym32_table(a.masks, g.nat, cell);
    const int st = lane < 27 ? int(tab[lane]) : 0;
    const unsigned slp = lane < 27 ? tab[27 + lane] : 0u;
    const int c = __popc(m);
    int ex = 0;
#pragma unroll
    for (int b = 0; b < 6; ++b) ex += __popc(__ballot_sync(0xffffffffu, (c >> b) & 1) & lt) << b;
    const int incl = ex + c;
    const int n = __shfl_sync(0xffffffffu, incl, 31);
    if (n != nexp) {
      if (lane == 0) atomicOr(a.err, kFlagInconsistent);
      continue;
    }
    if (base < 0 || base + n > a.capacity) {
      if (lane == 0) atomicOr(a.err, kFlagCapacity);
      continue;
    }
    for (int r0 = 0; r0 < n; r0 += 32) {
      const int r = r0 + lane;
      const int rr = min(r, n - 1);
      int q = 0;  // first stencil cell whose inclusive count exceeds rr
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int v = __shfl_sync(0xffffffffu, incl, q + step - 1);
        if (v <= rr) q += step;
      }
      const unsigned mq = __shfl_sync(0xffffffffu, m, q);
      const int exq = __shfl_sync(0xffffffffu, ex, q);
      const int stq = __shfl_sync(0xffffffffu, st, q);
      const unsigned slq = __shfl_sync(0xffffffffu, slp, q);
      if (r < n) {
        const int js = stq + kth_bit32(mq, rr - exq);
        const float4 rj = a.rec[js];
        const unsigned mj = __float_as_uint(rj.w);
        const int S0 = tag_s(slq, 0) + wi0 - (field10(mj, 0) - kW32Bias);
        const int S1 = tag_s(slq, 1) + wi1 - (field10(mj, 1) - kW32Bias);
        const int S2 = tag_s(slq, 2) + wi2 - (field10(mj, 2) - kW32Bias);
        const float R0 = fadd(fsub(rj.x, ri.x), cts32(g.C, S0, S1, S2, 0));
        const float R1 = fadd(fsub(rj.y, ri.y), cts32(g.C, S0, S1, S2, 1));
        const float R2 = fadd(fsub(rj.z, ri.z), cts32(g.C, S0, S1, S2, 2));
        const long long pos = base + r;
        a.oi[pos] = iid;
        a.oj[pos] = a.perm[js];
        a.oS[3 * pos + 0] = TI(S0);
        a.oS[3 * pos + 1] = TI(S1);
        a.oS[3 * pos + 2] = TI(S2);
        if (a.oR) {
          a.oR[3 * pos + 0] = R0;
          a.oR[3 * pos + 1] = R1;
          a.oR[3 * pos + 2] = R2;
        }
      }
    }
  }
}

// _getR (cell_list.jl:525-531) with T = Float32 over a whole list: R =
// (xj - xi) + C'S with the single-precision operations of the pair passes.
template <typename TI>
__global__ void __launch_bounds__(256) k_pair_vectors32(Geo32 g, const float* __restrict__ X,
                                                        const TI* __restrict__ pi, const TI* __restrict__ pj,
                                                        const TI* __restrict__ pS, long long npairs,
                                                        float* __restrict__ R) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npairs;
       p += (long long)gridDim.x * blockDim.x) {
    const long long i = min(max((long long)pi[p] - 1, 0LL), (long long)g.nat - 1);
    const long long j = min(max((long long)pj[p] - 1, 0LL), (long long)g.nat - 1);
    const int s0 = int(pS[3 * p + 0]), s1 = int(pS[3 * p + 1]), s2 = int(pS[3 * p + 2]);
#pragma unroll
    for (int k = 0; k < 3; ++k) R[3 * p + k] = fadd(fsub(X[3 * j + k], X[3 * i + k]), cts32(g.C, s0, s1, s2, k));
  }
}

// Largest squared displacement in FP32 (the Verlet skin test); NaN wins.
__global__ void __launch_bounds__(256) k_max_disp_sq32(const float* __restrict__ X, const float* __restrict__ Xref,
                                                       long long nat, unsigned* __restrict__ out) {
  float m = 0.f;
  for (long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x; a < nat; a += (long long)gridDim.x * blockDim.x) {
    const float d0 = X[3 * a + 0] - Xref[3 * a + 0], d1 = X[3 * a + 1] - Xref[3 * a + 1],
                d2 = X[3 * a + 2] - Xref[3 * a + 2];
    const float d = d0 * d0 + d1 * d1 + d2 * d2;
    m = (d > m || d != d) ? d : m;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float v = __shfl_xor_sync(0xffffffffu, m, o);
    m = (v > m || v != v) ? v : m;
  }
  // non-negative floats (and NaN) order like their bit patterns
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

}  // namespace

template <typename TI>
void launch_pair_vectors32(const Geo32& g, const float* X, const TI* pi, const TI* pj, const TI* pS, long long npairs,
                           float* R, int num_sms, cudaStream_t st) {
  if (npairs <= 0) return;
  k_pair_vectors32<TI><<<grid_for(npairs, 256, num_sms * 8), 256, 0, st>>>(g, X, pi, pj, pS, npairs, R);
}

void launch_max_disp_sq32(const float* X, const float* Xref, long long nat, unsigned* out, int num_sms,
                          cudaStream_t st) {
  if (nat <= 0) return;
  k_max_disp_sq32<<<grid_for(nat, 256, num_sms * 8), 256, 0, st>>>(X, Xref, nat, out);
}

void launch_bin32(const Geo32& g, const float* X, int nat, int* cid, int* ticket, float4* rec, int* cell_count,
                  unsigned* err, int num_sms, cudaStream_t st) {
  if (nat <= 0) return;
  k_bin32<false><<<grid_for(nat, 256, num_sms * 8), 256, 0, st>>>(g, nullptr, nullptr, nullptr, 0, X, nat, cid, ticket,
                                                                   rec, cell_count, err);
}

void launch_bin32_batch(const Geo32* geos, const int* atom0, const int* cell0, int nsys, const float* X, int nat,
                        int* cid, int* ticket, float4* rec, int* cell_count, unsigned* err, int num_sms,
                        cudaStream_t st) {
  if (nat <= 0 || nsys <= 0) return;
  Geo32 g0;
  memset(&g0, 0, sizeof(g0));
  k_bin32<true><<<grid_for(nat, 256, num_sms * 8), 256, 0, st>>>(g0, geos, atom0, cell0, nsys, X, nat, cid, ticket,
                                                                  rec, cell_count, err);
}

template <typename TI>
void launch_prepare32(const Geo32& g, const float* Xs, const TI* cell_id, const TI* perm, int nat, float4* rec_sorted,
                      int* scell, unsigned* err, int num_sms, cudaStream_t st) {
  if (nat <= 0) return;
  k_prepare32<TI><<<grid_for(nat, 256, num_sms * 8), 256, 0, st>>>(g, Xs, cell_id, perm, nat, rec_sorted, scell, err);
}

template <typename TI>
void launch_pairs32(bool fill, const Pairs32Args<TI>& a, int num_sms, cudaStream_t st) {
  if (a.nsys > 0) {  // batches: the per-cell passes (count, then the screening fill)
    if (a.nat_total <= 0 || a.ncells_total <= 0) return;
    const int grid = grid_for(a.ncells_total, kW32Warps, num_sms * 12);
    Pairs32Args<TI> r = a;
    r.round_pass = 1;
    if (fill) {
      k_pairs32<TI, true, true><<<grid, kW32Warps * 32, 0, st>>>(a);
      if (a.rounds) k_pairs32<TI, true, true><<<grid, kW32Warps * 32, 0, st>>>(r);
    } else {
      k_pairs32<TI, false, true><<<grid, kW32Warps * 32, 0, st>>>(a);
      if (a.rounds) k_pairs32<TI, false, true><<<grid, kW32Warps * 32, 0, st>>>(r);
    }
    return;
  }
  if (a.g.nat <= 0) return;
  const int grid = grid_for(a.g.ncells, kW32Warps, num_sms * 12);
  if (fill) {
    k_emit32_masks<TI><<<grid_for(a.g.nat, 4, num_sms * 16), 128, 0, st>>>(a);
    k_pairs32<TI, true, false><<<grid, kW32Warps * 32, 0, st>>>(a);
  } else {
    if (a.sym) k_pairs32_sym<TI><<<grid_for(a.g.ncells, kSym32Warps, num_sms * 16), kSym32Warps * 32, 0, st>>>(a);
    k_pairs32<TI, false, false><<<grid, kW32Warps * 32, 0, st>>>(a);
  }
}

#define NL_INST(TI)                                                                                                 \
  template void launch_prepare32<TI>(const Geo32&, const float*, const TI*, const TI*, int, float4*, int*,         \
                                     unsigned*, int, cudaStream_t);                                                \
  template void launch_pairs32<TI>(bool, const Pairs32Args<TI>&, int, cudaStream_t);                              \
  template void launch_pair_vectors32<TI>(const Geo32&, const float*, const TI*, const TI*, const TI*, long long,   \
                                          float*, int, cudaStream_t);
NL_INST(int32_t)
NL_INST(int64_t)
#undef NL_INST

}  // namespace nl
