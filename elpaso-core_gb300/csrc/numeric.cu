// K3 (per-w combine), K4/K7 (multifrontal numeric LU), K5 (triangular
// solves) and K6 (FP64 residual + refinement) for the complex dynamic
// stiffness system A(w) u = f.
//
// The reference solves each w with MUMPS (KSPPREONLY + PCLU,
// analysis/analysis.cpp:1159-1169, 1293-1332) on m_K after
// MatZeroRows(diag = 1) (analysis.cpp:419-454). Here:
//  - A(w) is formed on the device from the w-independent arrays (entry
//    classes, model.hpp), BC rows included, and scaled symmetrically by
//    D = diag(1/sqrt|a_ii|) so that pivots are O(1) in FP32 and FP64 alike;
//  - fronts are factorised level by level (all fronts of a level, and all
//    frequencies of a batch, in the same launches) with a right-looking
//    blocked LU: panel (partial pivoting restricted to the fully summed
//    rows, static-pivot floor for tiny pivots), border rows of the panel
//    (L21), pivot block row (U12), and the Schur update of the trailing
//    matrix -- complex GEMM, precision of the fronts;
//  - the Schur complement is extend-added into the parent, one child slot at
//    a time so the summation order is fixed (results do not depend on the
//    batch a frequency lands in);
//  - the residual r = f - A(w) x is always FP64 from the FP64 value arrays,
//    the correction is solved with the front-precision factors, and x is
//    updated in FP64 until ||r||/||f|| <= tol.
#include <algorithm>
#include <mutex>
#include <type_traits>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>

#include "numeric.cuh"
#include "prof.cuh"

namespace elp {

// ------------------------------------------------------------- complex ops
template <class R> struct Vec2;
template <> struct Vec2<double> { using T = double2; };
template <> struct Vec2<float> { using T = float2; };

__device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ float2 mkf(float a, float b) { return make_float2(a, b); }
template <class V> __device__ __forceinline__ V cmk(double a, double b);
template <> __device__ __forceinline__ double2 cmk<double2>(double a, double b) { return make_double2(a, b); }
template <> __device__ __forceinline__ float2 cmk<float2>(double a, double b) { return make_float2((float)a, (float)b); }

template <class V> __device__ __forceinline__ V cadd(V a, V b) { a.x += b.x; a.y += b.y; return a; }
template <class V> __device__ __forceinline__ V csub(V a, V b) { a.x -= b.x; a.y -= b.y; return a; }
template <class V> __device__ __forceinline__ V cmul(V a, V b) {
  V r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
// a - b * c
template <class V> __device__ __forceinline__ V cfms(V a, V b, V c) {
  a.x -= b.x * c.x - b.y * c.y;
  a.y -= b.x * c.y + b.y * c.x;
  return a;
}
// c + a * b
template <class V> __device__ __forceinline__ V cfma(V a, V b, V c) {
  c.x += a.x * b.x - a.y * b.y;
  c.y += a.x * b.y + a.y * b.x;
  return c;
}
template <class V> __device__ __forceinline__ auto cabs2(V a) -> decltype(a.x) { return a.x * a.x + a.y * a.y; }
template <class V> __device__ __forceinline__ V cinv(V a) {
  auto d = a.x * a.x + a.y * a.y;
  V r;
  r.x = a.x / d;
  r.y = -a.y / d;
  return r;
}

// ------------------------------------------------------------- combine

// F_s += G / w_s: the normal-velocity loads of each slot's right-hand side
__global__ void k_add_vn(const double2* __restrict__ g, const Coef* __restrict__ coef, int64_t n,
                         double2* __restrict__ f) {
  const int s = blockIdx.y;
  const double iw = coef[s].inv_w;
  double2* fs = f + s * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = g[i];
    if (v.x != 0.0 || v.y != 0.0) fs[i] = make_double2(fs[i].x + v.x * iw, fs[i].y + v.y * iw);
  }
}

// A group's right-hand sides: F(w) = F + G / w of each member at its own
// frequency of the slot, scaled to unit norm (fscale) so that the group's
// residual bounds every member's relative residual (G may be null)
__global__ void k_group_rhs(CombineArgs A, const double2* __restrict__ rhs, const double2* __restrict__ g,
                            const Coef* __restrict__ coef, int64_t n, double2* __restrict__ f) {
  const int s = blockIdx.y;
  double2* fs = f + s * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const Coef& c = row_coef(A, coef, s, i);
    double2 v = rhs[i];
    if (g) {
      const double2 t = g[i];
      if (t.x != 0.0 || t.y != 0.0) v = make_double2(v.x + t.x * c.inv_w, v.y + t.y * c.inv_w);
    }
    fs[i] = make_double2(v.x * c.fscale, v.y * c.fscale);
  }
}

// x of each group member back to its own right-hand side's scale
__global__ void k_group_unscale(CombineArgs A, const Coef* __restrict__ coef, int64_t n, double2* __restrict__ x) {
  const int s = blockIdx.y;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double d = 1.0 / row_coef(A, coef, s, i).fscale;
    const double2 v = x[s * n + i];
    x[s * n + i] = make_double2(v.x * d, v.y * d);
  }
}

// ||r||^2 and ||f||^2 of each group member in each slot (its rows are
// contiguous: [off[k], off[k + 1])), summed in a fixed order
__global__ void k_member_norms(const int64_t* __restrict__ off, int nm, int64_t n, const double2* __restrict__ r,
                               const double2* __restrict__ f, double* __restrict__ out) {
  const int k = blockIdx.x, s = blockIdx.y;
  double rr = 0.0, ff = 0.0;
  for (int64_t i = off[k] + threadIdx.x; i < off[k + 1]; i += blockDim.x) {
    const double2 a = r[s * n + i], b = f[s * n + i];
    rr += a.x * a.x + a.y * a.y;
    ff += b.x * b.x + b.y * b.y;
  }
  __shared__ double sr[256], sf[256];
  sr[threadIdx.x] = rr;
  sf[threadIdx.x] = ff;
  __syncthreads();
  for (int o = blockDim.x / 2; o; o >>= 1) {
    if ((int)threadIdx.x < o) { sr[threadIdx.x] += sr[threadIdx.x + o]; sf[threadIdx.x] += sf[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { out[2 * ((int64_t)s * nm + k)] = sr[0]; out[2 * ((int64_t)s * nm + k) + 1] = sf[0]; }
}

// residual rows of the group members that reached the tolerance set to zero:
// A and the preconditioner are block diagonal, so those members' solutions
// stop changing while the others go on
__global__ void k_mask_members(const int32_t* __restrict__ row_model, const int* __restrict__ done, int nm,
                               int64_t n, double2* __restrict__ r, const int* __restrict__ active) {
  const int s = blockIdx.y;
  if (!active[s]) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (done[(int64_t)s * nm + row_model[i]]) r[s * n + i] = make_double2(0.0, 0.0);
}

__global__ void k_dscale(CombineArgs A, const Coef* __restrict__ coef, const int32_t* __restrict__ diag,
                         int64_t n, double* __restrict__ dscale) {
  const int s = blockIdx.y;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double2 v = combine(A, row_coef(A, coef, s, i), diag[i]);
    double a = sqrt(v.x * v.x + v.y * v.y);
    dscale[s * n + i] = a > 0.0 ? 1.0 / sqrt(a) : 1.0;
  }
}

// A(w) values on the pattern (unscaled), for parity checks
__global__ void k_values(CombineArgs A, const Coef* __restrict__ coef, double2* __restrict__ out) {
  const Coef c = coef[0];
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < A.nnz; q += (int64_t)gridDim.x * blockDim.x)
    out[q] = combine(A, c, q);
}

// Full fronts starting at a level: zeroed in the front pool (their region
// may have held fronts that ended at an earlier level).
template <class V>
__global__ void k_zero_fronts(const int32_t* __restrict__ list, const int32_t* __restrict__ fp,
                              const int32_t* __restrict__ fb, const int64_t* __restrict__ foff,
                              V* __restrict__ pool, int64_t pool_size) {
  const int f = list[blockIdx.x];
  const int64_t m = (int64_t)fp[f] + fb[f], mm = m * m;
  V* F = pool + blockIdx.y * pool_size + foff[f];
  const int64_t t0 = blockIdx.z * (int64_t)blockDim.x + threadIdx.x, nt = (int64_t)gridDim.z * blockDim.x;
  // 16-byte stores: one 8-byte entry first when the front starts between 16-byte
  // boundaries (FP32 complex), the last one alone when an odd count remains
  const int64_t head = (sizeof(V) == 8 && (reinterpret_cast<uintptr_t>(F) & 15)) ? 1 : 0;
  const int64_t per16 = 16 / sizeof(V);
  const int64_t nq = (mm - head) / per16;
  float4* Q = reinterpret_cast<float4*>(F + head);
  for (int64_t t = t0; t < nq; t += nt) Q[t] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (t0 == 0) {
    const V z = cmk<V>(0.0, 0.0);
    if (head && mm > 0) F[0] = z;
    for (int64_t k = head + nq * per16; k < mm; ++k) F[k] = z;
  }
}

// A(w) entries owned by the fronts starting at a level, scaled by D on both
// sides, written into those fronts (every entry has one owner slot; entries
// in Dirichlet columns stay zero: the solve lifts them to the right-hand side)
template <class V>
__global__ void k_scatter(CombineArgs A, const Coef* __restrict__ coef, const int32_t* __restrict__ order,
                          int64_t count, const int32_t* __restrict__ entry_row, const int32_t* __restrict__ col_idx,
                          const int32_t* __restrict__ entry_owner, const int64_t* __restrict__ entry_local,
                          const int64_t* __restrict__ foff, const double* __restrict__ dscale, int64_t n,
                          V* __restrict__ pool, int64_t pool_size, unsigned long long* __restrict__ stats) {
  const int s = blockIdx.y;
  const double* d = dscale + s * n;
  V* F = pool + s * pool_size;
  double amax = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t q = order[t];
    if (A.cls[q] & CLS_BC_COLUMN) continue;
    const int32_t i = entry_row[q];
    double2 v = combine(A, row_coef(A, coef, s, i), q);
    const double sc = d[i] * d[col_idx[q]];
    v.x *= sc;
    v.y *= sc;
    amax = fmax(amax, sqrt(v.x * v.x + v.y * v.y));
    F[foff[entry_owner[q]] + entry_local[q]] = cmk<V>(v.x, v.y);
  }
  for (int o = 16; o; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  if ((threadIdx.x & 31) == 0) atomicMax(stats + 4 * s + 3, (unsigned long long)__double_as_longlong(amax));
}

// Factors of a level's fronts copied from the front pool into the factor
// store once the level is done: the m x p panel (contiguous, ld m) and U12
// (rows 0..p-1 of columns p..m-1) repacked with ld p.
template <class V>
__global__ void k_compact(const int32_t* __restrict__ list, const int32_t* __restrict__ fp,
                          const int32_t* __restrict__ fb, const int64_t* __restrict__ foff,
                          const int64_t* __restrict__ ffac, const V* __restrict__ pool, int64_t pool_size,
                          V* __restrict__ fac, int64_t fac_size) {
  const int f = list[blockIdx.x];
  const int64_t p = fp[f], b = fb[f], m = p + b;
  const V* src = pool + blockIdx.y * pool_size + foff[f];
  V* dst = fac + blockIdx.y * fac_size + ffac[f];
  const int64_t np = p * m, total = np + p * b;
  for (int64_t t = blockIdx.z * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.z * blockDim.x) {
    if (t < np) {
      dst[t] = src[t];
    } else {
      const int64_t u = t - np, i = u / p, r = u - i * p;
      dst[t] = src[(p + i) * m + r];
    }
  }
}

// ------------------------------------------------------------- panel
struct LevelArgs {
  const int32_t* list;      // fronts of the level (offset applied)
  int count;
  const int32_t *fp, *fb, *piv_off;
  const int64_t* foff;
  int64_t arena_size;
  int64_t n;
  // Schur complement added straight into the parent (extend-add fused into the
  // update; `list` then holds fronts with distinct parents)
  const int32_t *fparent, *map_off, *pmap;
  int fuse;
};

constexpr int kPanelSmemBytes = 200 * 1024;  // panel rows held in shared memory when they fit

// swap map of one panel per (front of the level, slot): [n, rows[2 NB], src[2 NB]],
// n = 0 when the panel interchanged no rows
template <int NB>
__host__ __device__ constexpr int swapmap_ints() { return 1 + 4 * NB; }

// Block-strided copy t = tid, tid + nt, ... < count with U loads in flight per
// thread: load(t) for U indices first, then store(t, value) for them, so the
// copy costs count / (nt U) memory latencies instead of count / nt. valid(t)
// masks entries that are neither loaded nor stored.
template <int U, class Valid, class Load, class Store>
__device__ __forceinline__ void staged_copy(int count, Valid valid, Load load, Store store) {
  const int nt = blockDim.x;
  for (int t0 = threadIdx.x; t0 < count; t0 += U * nt) {
    decltype(load(0)) v[U];
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (t0 + u * nt < count && valid(t0 + u * nt)) v[u] = load(t0 + u * nt);
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (t0 + u * nt < count && valid(t0 + u * nt)) store(t0 + u * nt, v[u]);
  }
}

// Panel factorisation (columns k0..k0+w-1, fully summed rows k0..p-1) with
// partial pivoting restricted to the fully summed rows and a static pivot
// floor. SMEM = true handles the fronts whose panel rows fit in shared memory
// (one load and one store of the panel instead of a memory round trip per
// column step; few registers, so many CTAs share an SM); SMEM = false the
// others, factorised in place with each row's loads issued together. Row interchanges are applied here to the
// panel columns only; the panel's net permutation of rows (at most 2 w rows)
// is written as a swap map that k_laswp applies to every other column.
template <class R, int NB, bool SMEM>
__global__ void __launch_bounds__(256) k_panel(LevelArgs L, typename Vec2<R>::T* __restrict__ arena,
                                               int32_t* __restrict__ perm, int step, R tiny,
                                               unsigned long long* __restrict__ stats, int32_t* __restrict__ swapmap,
                                               int cap_rows) {
  using V = typename Vec2<R>::T;
  extern __shared__ unsigned char psm_raw[];
  const int f = L.list[blockIdx.x];
  const int s = blockIdx.y;
  const int p = L.fp[f], m = p + L.fb[f];
  const int k0 = step * NB;
  if (k0 >= p) return;
  const int w = min(NB, p - k0);
  const int rows = p - k0;
  V* F = arena + s * L.arena_size + L.foff[f];
  int32_t* pv = perm + s * L.n + L.piv_off[f];
  __shared__ R red_v[8];
  __shared__ int red_i[8];
  __shared__ V prow[NB];
  __shared__ int s_piv, spiv[NB];
  __shared__ int s_rows[2 * NB], s_src[2 * NB], s_n;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if ((rows <= cap_rows) != SMEM) return;  // the other variant's front (uniform per CTA)
  // perm holds the front's row position map: row r of the factorised pivot
  // block is original row pv[r]; identity before the first panel, each panel
  // applies its swap map to it (below)
  if (step == 0)
    for (int r = tid; r < p; r += blockDim.x) pv[r] = r;
  constexpr bool in_smem = SMEM;
  V* P;       // P[c * ld + r] = F[(k0 + c) * m + k0 + r]
  int64_t ld;
  if (in_smem) {
    P = reinterpret_cast<V*>(psm_raw);
    ld = rows;
    staged_copy<4>(
        rows * w, [](int) { return true; },
        [&](int t) { const int c = t / rows, r = t - c * rows; return F[(int64_t)(k0 + c) * m + k0 + r]; },
        [&](int t, V v) { P[t] = v; });
    __syncthreads();
  } else {
    P = F + (int64_t)k0 * m + k0;
    ld = m;
  }
  int nstatic = 0;
  R pmax = 0, pmin = (R)1e30;
  for (int j = 0; j < w; ++j) {
    // ---- pivot search over the fully summed rows j..rows-1
    R best = -1;
    int bi = j;  // stays in range even when the whole column is NaN
    for (int r = j + tid; r < rows; r += blockDim.x) {
      R a = cabs2(P[j * ld + r]);
      if (a > best) { best = a; bi = r; }
    }
    for (int o = 16; o; o >>= 1) {
      R ob = __shfl_xor_sync(0xffffffffu, best, o);
      int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if (lane == 0) { red_v[wid] = best; red_i[wid] = bi; }
    __syncthreads();
    if (tid == 0) {
      R b0 = red_v[0];
      int i0 = red_i[0];
      for (int q = 1; q < (int)(blockDim.x >> 5); ++q)
        if (red_v[q] > b0 || (red_v[q] == b0 && red_i[q] < i0)) { b0 = red_v[q]; i0 = red_i[q]; }
      if (i0 < j || i0 >= rows) i0 = j;
      s_piv = i0;
      spiv[j] = k0 + i0;
    }
    __syncthreads();
    const int pr = s_piv;
    if (pr != j)
      for (int c = tid; c < w; c += blockDim.x) {
        V t = P[c * ld + j];
        P[c * ld + j] = P[c * ld + pr];
        P[c * ld + pr] = t;
      }
    __syncthreads();
    V d = P[j * ld + j];
    R ad = sqrt(cabs2(d));
    if (!(ad >= tiny)) {  // static pivot floor (also catches NaN); uniform over the CTA
      d = cmk<V>((double)tiny, 0.0);
      ad = tiny;
      ++nstatic;
      __syncthreads();
      if (tid == 0) P[j * ld + j] = d;
    }
    pmax = ad > pmax ? ad : pmax;
    pmin = ad < pmin ? ad : pmin;
    for (int c = j + 1 + tid; c < w; c += blockDim.x) prow[c] = P[c * ld + j];
    __syncthreads();
    const V inv = cinv(d);
    for (int r = j + 1 + tid; r < rows; r += blockDim.x) {
      const V l = cmul(P[j * ld + r], inv);
      P[j * ld + r] = l;
      if (in_smem) {
        for (int c = j + 1; c < w; ++c) P[c * ld + r] = cfms(P[c * ld + r], l, prow[c]);
      } else {
#pragma unroll
        for (int h = 0; h < NB; h += 16) {  // the row's panel entries right of the pivot, 16 loads together
          V a[16];
#pragma unroll
          for (int c = 0; c < 16; ++c)
            if (h + c > j && h + c < w) a[c] = P[(h + c) * ld + r];
#pragma unroll
          for (int c = 0; c < 16; ++c)
            if (h + c > j && h + c < w) P[(h + c) * ld + r] = cfms(a[c], l, prow[h + c]);
        }
      }
    }
    __syncthreads();
  }
  if (in_smem)
    staged_copy<4>(
        rows * w, [](int) { return true; }, [&](int t) { return P[t]; },
        [&](int t, V v) { const int c = t / rows, r = t - c * rows; F[(int64_t)(k0 + c) * m + k0 + r] = v; });
  if (tid == 0) {
    if (nstatic) atomicAdd(stats + 4 * s + 0, (unsigned long long)nstatic);
    atomicMax(stats + 4 * s + 1, (unsigned long long)__double_as_longlong((double)pmax));
    // min |u_jj| stored as bits of 1/|u_jj| max
    atomicMax(stats + 4 * s + 2, (unsigned long long)__double_as_longlong(1.0 / (double)pmin));
    // swap map: panel rows sit at list position row - k0, rows below the panel are appended
    int* mrows = s_rows;
    int* msrc = s_src;
    int n = w;
    bool any = false;
    for (int j = 0; j < w; ++j) { mrows[j] = k0 + j; msrc[j] = k0 + j; }
    for (int j = 0; j < w; ++j) {
      const int r = spiv[j];
      if (r == k0 + j) continue;
      any = true;
      int b = r - k0;
      if (b >= w) {
        b = -1;
        for (int q = w; q < n; ++q)
          if (mrows[q] == r) b = q;
        if (b < 0) { mrows[n] = r; msrc[n] = r; b = n++; }
      }
      const int t = msrc[j]; msrc[j] = msrc[b]; msrc[b] = t;
    }
    s_n = any ? n : 0;
  }
  __syncthreads();
  const int n = s_n;
  int32_t* mp = swapmap + ((int64_t)blockIdx.x * gridDim.y + s) * swapmap_ints<NB>();
  if (tid == 0) mp[0] = n;
  int32_t moved = 0;
  if (tid < n) {  // n <= 2 NB <= blockDim.x
    mp[1 + tid] = s_rows[tid];
    mp[1 + 2 * NB + tid] = s_src[tid];
    moved = pv[s_src[tid]];
  }
  __syncthreads();  // every source entry of the position map is read before any is overwritten
  if (tid < n) pv[s_rows[tid]] = moved;
}

// Row interchanges of one panel applied to every column outside it (LAPACK's
// laswp), from the panel's swap map (new[rows_i] = old[src_i], at most 2 NB
// rows). A warp moves one column: lane i handles list entries i and i + 32;
// all loads come before __syncwarp and all stores after it, since a source
// row may be another entry's destination. A CTA covers kLaswpCols columns.
constexpr int kLaswpCols = 64;
template <class R, int NB>
__global__ void __launch_bounds__(256) k_laswp(LevelArgs L, typename Vec2<R>::T* __restrict__ arena,
                                               const int32_t* __restrict__ swapmap, int step) {
  static_assert(NB <= 32, "two list entries per lane");
  using V = typename Vec2<R>::T;
  const int f = L.list[blockIdx.x];
  const int s = blockIdx.y;
  const int p = L.fp[f], m = p + L.fb[f];
  const int k0 = step * NB;
  if (k0 >= p) return;
  const int w = min(NB, p - k0);
  const int c0 = blockIdx.z * kLaswpCols;
  if (c0 >= m - w) return;
  const int32_t* mp = swapmap + ((int64_t)blockIdx.x * gridDim.y + s) * swapmap_ints<NB>();
  const int n = mp[0];
  if (n == 0) return;  // no interchange in this panel
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int r0 = lane < n ? mp[1 + lane] : 0, s0 = lane < n ? mp[1 + 2 * NB + lane] : 0;
  const int r1 = lane + 32 < n ? mp[1 + lane + 32] : 0, s1 = lane + 32 < n ? mp[1 + 2 * NB + lane + 32] : 0;
  V* F = arena + s * L.arena_size + L.foff[f];
  for (int cc = c0 + wid; cc < min(c0 + kLaswpCols, m - w); cc += blockDim.x >> 5) {
    const int c = cc < k0 ? cc : cc + w;  // columns outside the panel
    V* col = F + (int64_t)c * m;
    V v0, v1;
    if (lane < n) v0 = col[s0];
    if (lane + 32 < n) v1 = col[s1];
    __syncwarp();
    if (lane < n) col[r0] = v0;
    if (lane + 32 < n) col[r1] = v1;
    __syncwarp();
  }
}

// L21 of the panel: rows p..m-1, panel columns (row-wise triangular solve with U of the panel)
template <class R, int NB>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 4 : 1) k_border(LevelArgs L, typename Vec2<R>::T* __restrict__ arena, int step) {
  using V = typename Vec2<R>::T;
  const int f = L.list[blockIdx.x];
  const int s = blockIdx.y;
  const int p = L.fp[f], b = L.fb[f], m = p + b;
  const int k0 = step * NB;
  if (k0 >= p) return;
  const int w = min(NB, p - k0);
  V* F = arena + s * L.arena_size + L.foff[f];
  __shared__ V U[NB][NB + 1];
  __shared__ V dinv[NB];
  staged_copy<8>(
      w * w, [&](int t) { return t % w <= t / w; }, [&](int t) { return F[(int64_t)(k0 + t / w) * m + k0 + t % w]; },
      [&](int t, V v) { U[t % w][t / w] = v; });
  __syncthreads();
  for (int j = threadIdx.x; j < w; j += blockDim.x) dinv[j] = cinv(U[j][j]);
  __syncthreads();
  for (int r = p + blockIdx.z * blockDim.x + threadIdx.x; r < m; r += gridDim.z * blockDim.x) {
    V v[NB];
#pragma unroll
    for (int j = 0; j < NB; ++j)
      if (j < w) v[j] = F[(int64_t)(k0 + j) * m + r];
    // column-oriented: once v[i] is final, every later v[j] is updated independently
    // (critical path of NB steps instead of a chain of NB^2/2 dependent FMAs)
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      if (i < w) {
        v[i] = cmul(v[i], dinv[i]);
#pragma unroll
        for (int j = i + 1; j < NB; ++j)
          if (j < w) v[j] = cfms(v[j], v[i], U[i][j]);
      }
    }
#pragma unroll
    for (int j = 0; j < NB; ++j)
      if (j < w) F[(int64_t)(k0 + j) * m + r] = v[j];
  }
}

// U12 of the panel rows: columns k0+w..m-1, unit-lower solve with L of the panel.
// The w x kUrowCols block goes through shared memory: loaded and stored with
// lanes along the panel rows (contiguous), solved by one thread per column.
template <class R>
__host__ __device__ constexpr int urow_cols() { return sizeof(R) == 4 ? 128 : 32; }

template <class R, int NB>
__global__ void __launch_bounds__(128) k_urow(LevelArgs L, typename Vec2<R>::T* __restrict__ arena, int step) {
  using V = typename Vec2<R>::T;
  constexpr int TC = urow_cols<R>();
  const int f = L.list[blockIdx.x];
  const int s = blockIdx.y;
  const int p = L.fp[f], m = p + L.fb[f];
  const int k0 = step * NB;
  if (k0 >= p) return;
  const int w = min(NB, p - k0);
  V* F = arena + s * L.arena_size + L.foff[f];
  __shared__ V Lp[NB][NB + 1];
  __shared__ V tile[TC][NB + 1];  // [column][panel row]
  staged_copy<8>(
      w * w, [&](int t) { return t % w > t / w; }, [&](int t) { return F[(int64_t)(k0 + t / w) * m + k0 + t % w]; },
      [&](int t, V v) { Lp[t % w][t / w] = v; });
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int cb = k0 + w + blockIdx.z * TC; cb < m; cb += gridDim.z * TC) {
    {  // the warp's columns, 4 loads in flight per lane
      constexpr int U = 4;
      for (int cc0 = wid; cc0 < TC; cc0 += U * nw) {
        V v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int cc = cc0 + u * nw, c = cb + cc;
          if (cc < TC && c < m && lane < w) v[u] = F[(int64_t)c * m + k0 + lane];
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int cc = cc0 + u * nw, c = cb + cc;
          if (cc < TC && c < m && lane < w) tile[cc][lane] = v[u];
        }
      }
    }
    __syncthreads();
    if ((int)threadIdx.x < TC && cb + (int)threadIdx.x < m) {
      V v[NB];
#pragma unroll
      for (int j = 0; j < NB; ++j)
        if (j < w) v[j] = tile[threadIdx.x][j];
#pragma unroll
      for (int j = 1; j < NB; ++j) {
        if (j < w) {
          V t = v[j];
#pragma unroll
          for (int i = 0; i < NB; ++i)
            if (i < j) t = cfms(t, Lp[j][i], v[i]);
          v[j] = t;
        }
      }
#pragma unroll
      for (int j = 0; j < NB; ++j)
        if (j < w) tile[threadIdx.x][j] = v[j];
    }
    __syncthreads();
    for (int cc = wid; cc < TC; cc += nw) {
      const int c = cb + cc;
      if (c < m && lane < w) F[(int64_t)c * m + k0 + lane] = tile[cc][lane];
    }
    __syncthreads();
  }
}

// Left-looking (Crout) updates of a front, complex GEMM C -= A B on
// sub-blocks of the same column-major front F (ld = m):
//   GM_COL   before panel k: F[k0:m, k0:k0+w]   -= F[k0:m, 0:k0]  F[0:k0, k0:k0+w]
//   GM_ROW   after panel k:  F[k0:k0+w, k0+w:m] -= F[k0:k0+w, 0:k0] F[0:k0, k0+w:m]
//   GM_SCHUR after the last: F[p:m, p:m]        -= F[p:m, 0:p]   F[0:p, p:m]
// Every output is read and written once per call, and the depth K grows to
// the number of eliminated pivots, instead of a rank-32 read-modify-write of
// the whole trailing matrix per panel.
enum GemmMode { GM_COL = 0, GM_ROW = 1, GM_SCHUR = 2 };

__device__ __forceinline__ bool gemm_block(int mode, int p, int m, int k0, int w, int& ra, int& M, int& ca, int& N,
                                           int& K) {
  if (mode == GM_COL) { ra = k0; M = m - k0; ca = k0; N = w; K = k0; }
  else if (mode == GM_ROW) { ra = k0; M = w; ca = k0 + w; N = m - k0 - w; K = k0; }
  else { ra = p; M = m - p; ca = p; N = m - p; K = p; }
  return M > 0 && N > 0 && K > 0;
}

template <class R, int NB, int TM, int TN>
__global__ void __launch_bounds__(256) k_gemm(LevelArgs L, typename Vec2<R>::T* __restrict__ arena, int step, int mode) {
  using V = typename Vec2<R>::T;
  constexpr int TX = TN / 4, TY = TM / 4;  // 256 threads, 4 x 4 outputs each
  static_assert(TX * TY == 256, "tile");
  const int f = L.list[blockIdx.x];
  const int s = blockIdx.y;
  const int p = L.fp[f], m = p + L.fb[f];
  const int k0 = step * NB;
  if (mode != GM_SCHUR && k0 >= p) return;
  const int w = min(NB, p - k0);
  int ra, M, ca, N, K;
  if (!gemm_block(mode, p, m, k0, w, ra, M, ca, N, K)) return;
  const int tiles_r = (M + TM - 1) / TM, tiles_c = (N + TN - 1) / TN;
  const int ntiles = tiles_r * tiles_c;
  V* F = arena + s * L.arena_size + L.foff[f];
  constexpr int KC = 16;  // k chunk staged in shared memory
  __shared__ R As_re[KC][TM], As_im[KC][TM];
  __shared__ R Bs_re[KC][TN], Bs_im[KC][TN];
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  for (int tile = blockIdx.z; tile < ntiles; tile += gridDim.z) {
    const int r0 = ra + (tile % tiles_r) * TM;
    const int c0 = ca + (tile / tiles_r) * TN;
    const int rend = ra + M, cend = ca + N;
    R acc_re[4][4], acc_im[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b2 = 0; b2 < 4; ++b2) { acc_re[a][b2] = 0; acc_im[a][b2] = 0; }
    for (int kc = 0; kc < K; kc += KC) {
      __syncthreads();
      for (int t = threadIdx.x; t < KC * TM; t += blockDim.x) {
        int k = t / TM, i = t % TM;
        V a = (kc + k < K && r0 + i < rend) ? F[(int64_t)(kc + k) * m + r0 + i] : cmk<V>(0.0, 0.0);
        As_re[k][i] = a.x;
        As_im[k][i] = a.y;
      }
      for (int t = threadIdx.x; t < KC * TN; t += blockDim.x) {
        int j = t / KC, kk = t % KC;
        V bv = (kc + kk < K && c0 + j < cend) ? F[(int64_t)(c0 + j) * m + kc + kk] : cmk<V>(0.0, 0.0);
        Bs_re[kk][j] = bv.x;
        Bs_im[kk][j] = bv.y;
      }
      __syncthreads();
      const int kend = min(KC, K - kc);
      for (int k = 0; k < kend; ++k) {
        R ar[4], ai[4], br[4], bi[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) { ar[a] = As_re[k][ty + TY * a]; ai[a] = As_im[k][ty + TY * a]; }
#pragma unroll
        for (int b2 = 0; b2 < 4; ++b2) { br[b2] = Bs_re[k][tx + TX * b2]; bi[b2] = Bs_im[k][tx + TX * b2]; }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b2 = 0; b2 < 4; ++b2) {
            acc_re[a][b2] += ar[a] * br[b2] - ai[a] * bi[b2];
            acc_im[a][b2] += ar[a] * bi[b2] + ai[a] * br[b2];
          }
      }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b2 = 0; b2 < 4; ++b2) {
        int r = r0 + ty + TY * a, c = c0 + tx + TX * b2;
        if (r < rend && c < cend) {
          V* dst = F + (int64_t)c * m + r;
          V v = *dst;
          v.x -= acc_re[a][b2];
          v.y -= acc_im[a][b2];
          *dst = v;
        }
      }
  }
}

}  // namespace elp
#include "gemm_tc.cuh"
namespace elp {

// extend-add of children's Schur complements into their parents
template <class R>
__global__ void __launch_bounds__(256) k_extend_add(const int32_t* __restrict__ list, const int32_t* __restrict__ fp,
                                                    const int32_t* __restrict__ fb, const int32_t* __restrict__ fparent,
                                                    const int32_t* __restrict__ map_off, const int64_t* __restrict__ foff,
                                                    const int32_t* __restrict__ pmap, typename Vec2<R>::T* __restrict__ arena,
                                                    int64_t arena_size) {
  using V = typename Vec2<R>::T;
  const int c = list[blockIdx.x];
  const int s = blockIdx.y;
  const int pc = fp[c], bc = fb[c], mc = pc + bc;
  const int P = fparent[c];
  const int mP = fp[P] + fb[P];
  const V* C = arena + s * arena_size + foff[c];
  V* PF = arena + s * arena_size + foff[P];
  const int32_t* mp = pmap + map_off[c];
  for (int i = threadIdx.x; i < bc; i += blockDim.x) {
    const int pi = mp[i];
    // 4 columns per pass: their loads are independent and in flight together
    for (int j = blockIdx.z * 4; j < bc; j += gridDim.z * 4) {
      V sv[4], dv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (j + q < bc) {
          sv[q] = C[(int64_t)(pc + j + q) * mc + pc + i];
          dv[q] = PF[(int64_t)mp[j + q] * mP + pi];
        }
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (j + q < bc) PF[(int64_t)mp[j + q] * mP + pi] = cadd(dv[q], sv[q]);
    }
  }
}

// ------------------------------------------------------------- solves
struct SolveArgs {
  const int32_t* list;
  int count;
  const int32_t *fp, *fb, *idx_off, *map_off, *cb_off, *piv_off, *child_ptr, *child_list;
  const int64_t* foff;
  const int32_t* dofs;
  const int32_t* pmap;
  int64_t arena_size, n, cb_total;
  const int* active;
  int u12_ld_p;  // U12 after the m x p panel with ld p (factor store), else in place with ld m
  // levels whose front vector does not fit shared memory: one global slice of
  // gvec_stride entries per (front of the level, slot), else null
  void* gvec;
  int64_t gvec_stride;
  // groups: fronts of (member, slot) pairs whose input rows are zero (pact 0)
  // are skipped -- their exact output is zero, which k_rhs already wrote
  const int32_t* fmember;
  const int* pact;
  int nm;
};

__device__ __forceinline__ bool front_skipped(const SolveArgs& S, int f, int s) {
  return S.pact && !S.pact[(int64_t)s * S.nm + S.fmember[f]];
}

// the sweep kernels' working vector: the CTA's global slice (G), or shared
// memory; a compile-time choice, so that the shared-memory variants address
// shared memory directly instead of through generic pointers
template <class V, bool G>
__device__ __forceinline__ V* solve_buf(const SolveArgs& S, unsigned char* smraw) {
  if (G) return reinterpret_cast<V*>(S.gvec) + ((int64_t)blockIdx.y * S.count + blockIdx.x) * S.gvec_stride;
  return reinterpret_cast<V*>(smraw);
}

// dst[k] = src[idx[k]] for k < count: every thread issues the index loads of
// four entries, then their value loads, so the dependent pairs of loads
// overlap instead of running one after another
template <class V>
__device__ __forceinline__ void gather_rows(V* dst, const V* __restrict__ src, const int32_t* __restrict__ idx,
                                            int count) {
  const int nt = blockDim.x;
  for (int k0 = threadIdx.x; k0 < count; k0 += 4 * nt) {
    int ix[4];
    V v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) ix[q] = k0 + q * nt < count ? idx[k0 + q * nt] : 0;
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (k0 + q * nt < count) v[q] = src[ix[q]];
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (k0 + q * nt < count) dst[k0 + q * nt] = v[q];
  }
}

template <class R, bool G>
__global__ void __launch_bounds__(512) k_forward(SolveArgs S, const typename Vec2<R>::T* __restrict__ arena,
                                                 const int32_t* __restrict__ perm, typename Vec2<R>::T* __restrict__ z,
                                                 typename Vec2<R>::T* __restrict__ cb) {
  using V = typename Vec2<R>::T;
  extern __shared__ unsigned char smraw[];
  V* w = solve_buf<V, G>(S, smraw);
  const int f = S.list[blockIdx.x];
  const int s = blockIdx.y;
  if (!S.active[s] || front_skipped(S, f, s)) return;
  const int p = S.fp[f], b = S.fb[f], m = p + b;
  const V* F = arena + s * S.arena_size + S.foff[f];
  const int32_t* I = S.dofs + S.idx_off[f];
  V* zs = z + s * S.n;
  V* cbs = cb + s * S.cb_total;
  const int tid = threadIdx.x;
  gather_rows(w, zs, I, p);
  for (int k = p + tid; k < m; k += blockDim.x) w[k] = cmk<V>(0.0, 0.0);
  __syncthreads();
  for (int q = S.child_ptr[f]; q < S.child_ptr[f + 1]; ++q) {
    const int c = S.child_list[q];
    const int bc = S.fb[c];
    const int32_t* mp = S.pmap + S.map_off[c];
    const V* src = cbs + S.cb_off[c];
    const int nt = blockDim.x;
    for (int i0 = tid; i0 < bc; i0 += 4 * nt) {  // four entries' loads in flight (targets are distinct)
      int mi[4];
      V sv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (i0 + u * nt < bc) { mi[u] = mp[i0 + u * nt]; sv[u] = src[i0 + u * nt]; }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (i0 + u * nt < bc) w[mi[u]] = cadd(w[mi[u]], sv[u]);
    }
    __syncthreads();
  }
  {  // row interchanges of the factorisation: pivot row j is original row pv[j]
    V* w2 = w + m;
    const int32_t* pv = perm + s * S.n + S.piv_off[f];
    for (int j = tid; j < p; j += blockDim.x) w2[j] = w[pv[j]];
    __syncthreads();
    for (int j = tid; j < p; j += blockDim.x) w[j] = w2[j];
    __syncthreads();
  }
  const int lane = tid & 31, wid = tid >> 5;
  // L11 solve on the pivot block only; the border rows (L21) are updated by
  // k_fwd_border across many CTAs
  __shared__ V dblk[32][33];  // diagonal 32 x 32 block, staged so the warp solve never waits on DRAM
  for (int j0 = 0; j0 < p; j0 += 32) {
    const int jw = min(32, p - j0);
    staged_copy<sizeof(R) == 4 ? 8 : 4>(
        32 * 32, [&](int t) { return (t >> 5) < jw && (t & 31) < jw; },
        [&](int t) { return F[(int64_t)(j0 + (t >> 5)) * m + j0 + (t & 31)]; },
        [&](int t, V v) { dblk[t & 31][t >> 5] = v; });
    __syncthreads();
    if (wid == 0) {
      V val = lane < jw ? w[j0 + lane] : cmk<V>(0.0, 0.0);
      for (int jj = 0; jj < jw; ++jj) {
        V x;
        x.x = __shfl_sync(0xffffffffu, val.x, jj);
        x.y = __shfl_sync(0xffffffffu, val.y, jj);
        if (lane > jj && lane < jw) val = cfms(val, dblk[lane][jj], x);
      }
      if (lane < jw) w[j0 + lane] = val;
    }
    __syncthreads();
    for (int r = j0 + jw + tid; r < p; r += blockDim.x) {
      V a[32];  // all loads of the row first: one memory latency per row, not 32
#pragma unroll
      for (int jj = 0; jj < 32; ++jj) a[jj] = jj < jw ? F[(int64_t)(j0 + jj) * m + r] : cmk<V>(0.0, 0.0);
      V t = w[r];
#pragma unroll
      for (int jj = 0; jj < 32; ++jj)
        if (jj < jw) t = cfms(t, a[jj], w[j0 + jj]);
      w[r] = t;
    }
    __syncthreads();
  }
  for (int k = tid; k < m; k += blockDim.x) {
    if (k < p) zs[I[k]] = w[k];
    else cbs[S.cb_off[f] + k - p] = w[k];
  }
}

// border rows of the forward step: cb -= L21 y_p. A CTA takes 32 border rows
// (lane = row, loads coalesced along the column); its 8 warps split the p
// columns and their partial sums are added in a fixed order.
template <class R, bool G>
__global__ void __launch_bounds__(256) k_fwd_border(SolveArgs S, const typename Vec2<R>::T* __restrict__ arena,
                                                    const typename Vec2<R>::T* __restrict__ z,
                                                    typename Vec2<R>::T* __restrict__ cb) {
  using V = typename Vec2<R>::T;
  extern __shared__ unsigned char smraw[];
  // global slices: the forward launch of this level left y_p in its first p entries
  V* y = solve_buf<V, G>(S, smraw);
  __shared__ V part[8][32];
  const int f = S.list[blockIdx.x];
  const int s = blockIdx.y;
  if (!S.active[s] || front_skipped(S, f, s)) return;
  const int p = S.fp[f], b = S.fb[f], m = p + b;
  if ((int)blockIdx.z * 32 >= b) return;
  const V* F = arena + s * S.arena_size + S.foff[f];
  const int32_t* I = S.dofs + S.idx_off[f];
  const V* zs = z + s * S.n;
  if (!G) gather_rows(y, zs, I, p);
  __syncthreads();
  const int lane = threadIdx.x & 31, wv = threadIdx.x >> 5;
  const int i = blockIdx.z * 32 + lane;
  V t = cmk<V>(0.0, 0.0);
  if (i < b) {
    const V* col = F + p + i;
    const int j_lo = (p * wv) / 8, j_hi = (p * (wv + 1)) / 8;
    int j = j_lo;
    for (; j + 16 <= j_hi; j += 16) {  // 16 independent loads in flight per thread
      V a[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) a[q] = col[(int64_t)(j + q) * m];
#pragma unroll
      for (int q = 0; q < 16; ++q) t = cfma(a[q], y[j + q], t);
    }
    for (; j < j_hi; ++j) t = cfma(col[(int64_t)j * m], y[j], t);
  }
  part[wv][lane] = t;
  __syncthreads();
  if (wv == 0 && i < b) {
    V sum = part[0][lane];
#pragma unroll
    for (int q = 1; q < 8; ++q) sum = cadd(sum, part[q][lane]);
    V* dst = cb + s * S.cb_total + S.cb_off[f] + i;
    *dst = csub(*dst, sum);
  }
}

// pivot rows of the backward step: t = y_p - U12 x_b. A CTA takes 32 pivot
// rows (lane = row); its 8 warps split the b border columns, partial sums
// added in a fixed order.
template <class R, bool G>
__global__ void __launch_bounds__(256) k_bwd_u12(SolveArgs S, const typename Vec2<R>::T* __restrict__ arena,
                                                 const typename Vec2<R>::T* __restrict__ z,
                                                 typename Vec2<R>::T* __restrict__ tb) {
  using V = typename Vec2<R>::T;
  extern __shared__ unsigned char smraw[];
  // global slices: k_gather_border filled the first b entries with x_b
  V* xb = solve_buf<V, G>(S, smraw);
  __shared__ V part[8][32];
  const int f = S.list[blockIdx.x];
  const int s = blockIdx.y;
  if (!S.active[s] || front_skipped(S, f, s)) return;
  const int p = S.fp[f], b = S.fb[f], m = p + b;
  if ((int)blockIdx.z * 32 >= p) return;
  const V* F = arena + s * S.arena_size + S.foff[f];
  const int32_t* I = S.dofs + S.idx_off[f];
  const V* zs = z + s * S.n;
  if (!G) gather_rows(xb, zs, I + p, b);
  __syncthreads();
  const int lane = threadIdx.x & 31, wv = threadIdx.x >> 5;
  const int r = blockIdx.z * 32 + lane;
  V t = cmk<V>(0.0, 0.0);
  if (r < p) {
    // U12 in place (row r of columns p..m-1, ld m), or in the factor store right
    // after the m x p panel with ld p: both start at F + p m + r
    const V* row = F + (int64_t)p * m + r;
    const int64_t ld = S.u12_ld_p ? p : m;
    const int i_lo = (b * wv) / 8, i_hi = (b * (wv + 1)) / 8;
    int i = i_lo;
    for (; i + 16 <= i_hi; i += 16) {  // 16 independent loads in flight per thread
      V a[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) a[q] = row[(int64_t)(i + q) * ld];
#pragma unroll
      for (int q = 0; q < 16; ++q) t = cfma(a[q], xb[i + q], t);
    }
    for (; i < i_hi; ++i) t = cfma(row[(int64_t)i * ld], xb[i], t);
  }
  part[wv][lane] = t;
  __syncthreads();
  if (wv == 0 && r < p) {
    V sum = part[0][lane];
#pragma unroll
    for (int q = 1; q < 8; ++q) sum = cadd(sum, part[q][lane]);
    tb[s * S.n + S.piv_off[f] + r] = csub(zs[I[r]], sum);
  }
}

// global slices only: x_b of each (front, slot) into the first b entries of
// its slice, once, for the k_bwd_u12 CTAs that share it
template <class R>
__global__ void __launch_bounds__(256) k_gather_border(SolveArgs S, const typename Vec2<R>::T* __restrict__ z) {
  using V = typename Vec2<R>::T;
  const int f = S.list[blockIdx.x];
  const int s = blockIdx.y;
  if (!S.active[s] || front_skipped(S, f, s)) return;
  const int p = S.fp[f], b = S.fb[f];
  V* xb = reinterpret_cast<V*>(S.gvec) + ((int64_t)blockIdx.y * S.count + blockIdx.x) * S.gvec_stride;
  gather_rows(xb, z + s * S.n, S.dofs + S.idx_off[f] + p, b);
}

template <class R, bool G>
__global__ void __launch_bounds__(512) k_backward(SolveArgs S, const typename Vec2<R>::T* __restrict__ arena,
                                                  typename Vec2<R>::T* __restrict__ z,
                                                  const typename Vec2<R>::T* __restrict__ tb) {
  using V = typename Vec2<R>::T;
  extern __shared__ unsigned char smraw[];
  V* w = solve_buf<V, G>(S, smraw);
  const int f = S.list[blockIdx.x];
  const int s = blockIdx.y;
  if (!S.active[s] || front_skipped(S, f, s)) return;
  const int p = S.fp[f], m = p + S.fb[f];
  const V* F = arena + s * S.arena_size + S.foff[f];
  const int32_t* I = S.dofs + S.idx_off[f];
  V* zs = z + s * S.n;
  const int tid = threadIdx.x;
  for (int k = tid; k < p; k += blockDim.x) w[k] = tb[s * S.n + S.piv_off[f] + k];
  __syncthreads();
  const int lane = tid & 31, wid = tid >> 5;
  __shared__ V dblk[32][33];  // diagonal 32 x 32 block, staged so the warp solve never waits on DRAM
  for (int jend = p; jend > 0; jend -= 32) {
    const int j0 = max(0, jend - 32);
    const int jw = jend - j0;
    staged_copy<sizeof(R) == 4 ? 8 : 4>(
        32 * 32, [&](int t) { return (t >> 5) < jw && (t & 31) < jw; },
        [&](int t) { return F[(int64_t)(j0 + (t >> 5)) * m + j0 + (t & 31)]; },
        [&](int t, V v) { dblk[t & 31][t >> 5] = v; });
    __syncthreads();
    if (wid == 0) {
      V val = lane < jw ? w[j0 + lane] : cmk<V>(0.0, 0.0);
      // every lane inverts its own diagonal entry up front: no division on the sequential chain
      const V dinv = lane < jw ? cinv(dblk[lane][lane]) : cmk<V>(0.0, 0.0);
      for (int jj = jw - 1; jj >= 0; --jj) {
        if (lane == jj) val = cmul(val, dinv);
        V x;
        x.x = __shfl_sync(0xffffffffu, val.x, jj);
        x.y = __shfl_sync(0xffffffffu, val.y, jj);
        if (lane < jj) val = cfms(val, dblk[lane][jj], x);
      }
      if (lane < jw) w[j0 + lane] = val;
    }
    __syncthreads();
    for (int r = tid; r < j0; r += blockDim.x) {
      V a[32];  // all loads of the row first: one memory latency per row, not 32
#pragma unroll
      for (int jj = 0; jj < 32; ++jj) a[jj] = jj < jw ? F[(int64_t)(j0 + jj) * m + r] : cmk<V>(0.0, 0.0);
      V t = w[r];
#pragma unroll
      for (int jj = 0; jj < 32; ++jj)
        if (jj < jw) t = cfms(t, a[jj], w[j0 + jj]);
      w[r] = t;
    }
    __syncthreads();
  }
  for (int k = tid; k < p; k += blockDim.x) zs[I[k]] = w[k];
}

// ------------------------------------------------------------- refinement (FP64)
// r = f - A x (unscaled A, BC rows included); partial sums of |r|^2 and |f|^2
// kRowLanes lanes per row; the row loop bound is warp-uniform so every lane
// reaches every shuffle. With x_zero the residual is f itself (no product).
__global__ void k_residual(CombineArgs A, const Coef* __restrict__ coef, const int32_t* __restrict__ row_ptr,
                           const int32_t* __restrict__ col_idx, int64_t n, const double2* __restrict__ x,
                           const double2* __restrict__ f, double2* __restrict__ r, double* __restrict__ partial,
                           int nparts, const int* __restrict__ active, int x_zero) {
  const int s = blockIdx.y;
  if (!active[s]) return;
  const int lane = threadIdx.x & 31, sub = lane & (kRowLanes - 1);
  const double2* xs = x + s * n;
  double rr = 0.0, ff = 0.0;
  constexpr int RPW = 32 / kRowLanes;  // rows per warp
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = warp * RPW; base < n; base += nwarps * RPW) {
    const int64_t i = base + lane / kRowLanes;
    // a group's finished pairs (A.pact) keep their residual rows: their x did not change
    const bool on = i < n && row_on(A, s, i);
    DD sx{0.0, 0.0}, sy{0.0, 0.0};
    if (on && !x_zero) {
      const Coef& c = row_coef(A, coef, s, i);
      for (int q = row_ptr[i] + sub; q < row_ptr[i + 1]; q += kRowLanes) {
        double2 a = combine(A, c, q);
        double2 v = xs[col_idx[q]];
        dd_fma(sx, a.x, v.x);
        dd_fma(sx, -a.y, v.y);
        dd_fma(sy, a.x, v.y);
        dd_fma(sy, a.y, v.x);
      }
    }
    if (!x_zero) {
      sx = row_sum(sx);
      sy = row_sum(sy);
    }
    if (on && sub == 0) {
      double2 fi = f[s * n + i];
      double2 ri = x_zero ? fi : make_double2(dd_residual(fi.x, sx), dd_residual(fi.y, sy));
      r[s * n + i] = ri;
      rr += ri.x * ri.x + ri.y * ri.y;
      ff += fi.x * fi.x + fi.y * fi.y;
    }
  }
  for (int o = 16; o; o >>= 1) {
    rr += __shfl_xor_sync(0xffffffffu, rr, o);
    ff += __shfl_xor_sync(0xffffffffu, ff, o);
  }
  __shared__ double red[2][32];
  const int wid = threadIdx.x >> 5;
  if (lane == 0) { red[0][wid] = rr; red[1][wid] = ff; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { a += red[0][q]; b += red[1][q]; }
    partial[(s * (int64_t)nparts + blockIdx.x) * 2 + 0] = a;
    partial[(s * (int64_t)nparts + blockIdx.x) * 2 + 1] = b;
  }
}

__global__ void k_norms(const double* __restrict__ partial, int nparts, double* __restrict__ norms,
                        const int* __restrict__ active) {
  const int s = blockIdx.x;
  if (!active[s]) return;
  __shared__ double a[256], b[256];
  double x = 0, y = 0;
  for (int q = threadIdx.x; q < nparts; q += blockDim.x) {
    x += partial[(s * (int64_t)nparts + q) * 2];
    y += partial[(s * (int64_t)nparts + q) * 2 + 1];
  }
  a[threadIdx.x] = x;
  b[threadIdx.x] = y;
  __syncthreads();
  for (int o = blockDim.x / 2; o; o >>= 1) {
    if ((int)threadIdx.x < o) { a[threadIdx.x] += a[threadIdx.x + o]; b[threadIdx.x] += b[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { norms[2 * s] = a[0]; norms[2 * s + 1] = b[0]; }
}

// z = D (r - A(:, bc) r_bc) in front precision (r of slot s at r + s * sstride):
// Dirichlet columns are lifted to the right-hand side (the factorisation
// holds A with those columns removed, and r_bc passes through the identity
// rows), so the preconditioner is the exact inverse of A up to the front
// precision.
template <class V>
__global__ void k_rhs(CombineArgs A, const Coef* __restrict__ coef, const int32_t* __restrict__ row_ptr,
                      const int32_t* __restrict__ col_idx, const double2* __restrict__ r, int64_t sstride,
                      const double* __restrict__ dscale, int64_t n, V* __restrict__ z, const int* __restrict__ active) {
  const int s = blockIdx.y;
  if (!active[s]) return;
  const int lane = threadIdx.x & 31, sub = lane & (kRowLanes - 1);
  const double2* rs = r + s * sstride;
  constexpr int RPW = 32 / kRowLanes;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = warp * RPW; base < n; base += nwarps * RPW) {
    const int64_t i = base + lane / kRowLanes;
    const bool on = i < n && row_on(A, s, i);
    double sx = 0.0, sy = 0.0;
    bool lift = false;  // entries in Dirichlet columns: lifted to the right-hand side
    if (on)
      for (int q = row_ptr[i] + sub; q < row_ptr[i + 1]; q += kRowLanes) {
        if (!(A.cls[q] & CLS_BC_COLUMN)) continue;
        lift = true;
        double2 a = combine(A, row_coef(A, coef, s, i), q);
        double2 v = rs[col_idx[q]];
        sx += a.x * v.x - a.y * v.y;
        sy += a.x * v.y + a.y * v.x;
      }
    if (__any_sync(0xffffffffu, lift)) {  // most rows touch no Dirichlet column
      sx = row_sum(sx);
      sy = row_sum(sy);
    }
    if (on && sub == 0) {
      const double d = dscale[s * n + i];
      const double2 v = rs[i];
      z[s * n + i] = cmk<V>((v.x - sx) * d, (v.y - sy) * d);
    }
  }
}

// x += D z
template <class V>
__global__ void k_update(double2* __restrict__ x, const double* __restrict__ dscale, int64_t n, const V* __restrict__ z,
                         const int* __restrict__ active) {
  const int s = blockIdx.y;
  if (!active[s]) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double d = dscale[s * n + i];
    V v = z[s * n + i];
    double2 t = x[s * n + i];
    t.x += d * (double)v.x;
    t.y += d * (double)v.y;
    x[s * n + i] = t;
  }
}

// ------------------------------------------------------------- GMRES (FP64)
// Right-preconditioned restarted GMRES on A(w) x = f, preconditioner
// M^-1 = D (LU)^-1 D with the front-precision factors. The Arnoldi vectors,
// the SpMV and the orthogonalisation (classical Gram-Schmidt, twice) are
// FP64; only the preconditioner solve runs in the front precision.
constexpr int kMaxBasis = 32;

// w = A u (FP64, unscaled A)
__global__ void k_spmv(CombineArgs A, const Coef* __restrict__ coef, const int32_t* __restrict__ row_ptr,
                       const int32_t* __restrict__ col_idx, int64_t n, const double2* __restrict__ u, int64_t ustride,
                       double2* __restrict__ w, const int* __restrict__ active) {
  const int s = blockIdx.y;
  if (!active[s]) return;
  const int lane = threadIdx.x & 31, sub = lane & (kRowLanes - 1);
  const double2* us = u + s * ustride;
  constexpr int RPW = 32 / kRowLanes;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = warp * RPW; base < n; base += nwarps * RPW) {
    const int64_t i = base + lane / kRowLanes;
    const bool on = i < n && row_on(A, s, i);
    double sx = 0.0, sy = 0.0;
    if (on) {
      const Coef& c = row_coef(A, coef, s, i);
      for (int q = row_ptr[i] + sub; q < row_ptr[i + 1]; q += kRowLanes) {
        double2 a = combine(A, c, q);
        double2 v = us[col_idx[q]];
        sx += a.x * v.x - a.y * v.y;
        sy += a.x * v.y + a.y * v.x;
      }
    }
    sx = row_sum(sx);
    sy = row_sum(sy);
    if (on && sub == 0) w[s * n + i] = make_double2(sx, sy);
  }
}

// partial[s][block][i] = sum_r conj(V_i[r]) w[r], V_i = basis + s*sstride + i*vstride
__global__ void k_dots(const double2* __restrict__ basis, int64_t sstride, int64_t vstride, int nv,
                       const double2* __restrict__ w, int64_t n, double2* __restrict__ partial, int nparts,
                       const int* __restrict__ active) {
  const int s = blockIdx.y;
  if (!active[s]) return;
  __shared__ double red[2][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const double2* ws = w + s * n;
  for (int i = 0; i < nv; ++i) {
    const double2* v = basis + s * sstride + (int64_t)i * vstride;
    double ax = 0.0, ay = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
      double2 a = v[r], b = ws[r];
      ax += a.x * b.x + a.y * b.y;
      ay += a.x * b.y - a.y * b.x;
    }
    for (int o = 16; o; o >>= 1) {
      ax += __shfl_xor_sync(0xffffffffu, ax, o);
      ay += __shfl_xor_sync(0xffffffffu, ay, o);
    }
    if (lane == 0) { red[0][wid] = ax; red[1][wid] = ay; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double tx = 0, ty = 0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { tx += red[0][q]; ty += red[1][q]; }
      partial[((int64_t)s * nparts + blockIdx.x) * kMaxBasis + i] = make_double2(tx, ty);
    }
    __syncthreads();
  }
}

// h[s][i] = sum over blocks (fixed order)
__global__ void k_dots_reduce(const double2* __restrict__ partial, int nparts, int nv, double2* __restrict__ h,
                              const int* __restrict__ active) {
  const int s = blockIdx.x;
  if (!active[s]) return;
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    double tx = 0, ty = 0;
    for (int b = 0; b < nparts; ++b) {
      double2 v = partial[((int64_t)s * nparts + b) * kMaxBasis + i];
      tx += v.x;
      ty += v.y;
    }
    h[s * kMaxBasis + i] = make_double2(tx, ty);
  }
}

// w -= sum_i h_i V_i ; accumulates h into hsum
__global__ void k_gs(const double2* __restrict__ basis, int64_t sstride, int64_t vstride, int nv,
                     const double2* __restrict__ h, double2* __restrict__ w, int64_t n, const int* __restrict__ active) {
  const int s = blockIdx.y;
  if (!active[s]) return;
  __shared__ double2 hs[kMaxBasis];
  if (threadIdx.x < nv) hs[threadIdx.x] = h[s * kMaxBasis + threadIdx.x];
  __syncthreads();
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double2 t = w[s * n + r];
    for (int i = 0; i < nv; ++i) {
      double2 v = basis[s * sstride + (int64_t)i * vstride + r];
      t.x -= hs[i].x * v.x - hs[i].y * v.y;
      t.y -= hs[i].x * v.y + hs[i].y * v.x;
    }
    w[s * n + r] = t;
  }
}

// dst = src * scale[s] (real scale from the host)
__global__ void k_vscale(const double2* __restrict__ src, double2* __restrict__ dst, int64_t sstride_dst,
                         const double* __restrict__ scale, int64_t n, const int* __restrict__ active) {
  const int s = blockIdx.y;
  if (!active[s]) return;
  const double a = scale[s];
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double2 v = src[s * n + r];
    dst[s * sstride_dst + r] = make_double2(v.x * a, v.y * a);
  }
}

// t += sum_i y_i Z_i
__global__ void k_combo(const double2* __restrict__ basis, int64_t sstride, int64_t vstride, int nv,
                        const double2* __restrict__ y, double2* __restrict__ t, int64_t n, const int* __restrict__ active) {
  const int s = blockIdx.y;
  if (!active[s]) return;
  __shared__ double2 ys[kMaxBasis];
  if (threadIdx.x < nv) ys[threadIdx.x] = y[s * kMaxBasis + threadIdx.x];
  __syncthreads();
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double ax = t[s * n + r].x, ay = t[s * n + r].y;
    for (int i = 0; i < nv; ++i) {
      double2 v = basis[s * sstride + (int64_t)i * vstride + r];
      ax += ys[i].x * v.x - ys[i].y * v.y;
      ay += ys[i].x * v.y + ys[i].y * v.x;
    }
    t[s * n + r] = make_double2(ax, ay);
  }
}

// ---- GMRES per group member: the same vector kernels, with one set of
// coefficients per (slot, member) pair p = s * nm + k (rows of member k are
// off[k] .. off[k + 1] - 1)

// out[p * kMaxBasis + i] = sum over member k's rows of conj(V_i) w, one CTA per pair (fixed order)
__global__ void k_dots_seg(const double2* __restrict__ basis, int64_t sstride, int64_t vstride, int nv,
                           const double2* __restrict__ w, int64_t wstride, const int64_t* __restrict__ off, int nm,
                           double2* __restrict__ out, const int* __restrict__ pact) {
  const int k = blockIdx.x, s = blockIdx.y;
  const int64_t p = (int64_t)s * nm + k;
  if (!pact[p]) return;
  __shared__ double red[2][256];
  const double2* ws = w + s * wstride;
  for (int i = 0; i < nv; ++i) {
    const double2* v = basis + s * sstride + (int64_t)i * vstride;
    double ax = 0.0, ay = 0.0;
    for (int64_t r = off[k] + threadIdx.x; r < off[k + 1]; r += blockDim.x) {
      const double2 a = v[r], b = ws[r];
      ax += a.x * b.x + a.y * b.y;
      ay += a.x * b.y - a.y * b.x;
    }
    red[0][threadIdx.x] = ax;
    red[1][threadIdx.x] = ay;
    __syncthreads();
    for (int o = blockDim.x / 2; o; o >>= 1) {
      if ((int)threadIdx.x < o) {
        red[0][threadIdx.x] += red[0][threadIdx.x + o];
        red[1][threadIdx.x] += red[1][threadIdx.x + o];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) out[p * kMaxBasis + i] = make_double2(red[0][0], red[1][0]);
    __syncthreads();
  }
}

// w -= sum_i h_{p,i} V_i on every row (its pair's coefficients)
__global__ void k_gs_seg(const double2* __restrict__ basis, int64_t sstride, int64_t vstride, int nv,
                         const double2* __restrict__ h, double2* __restrict__ w, int64_t n,
                         const int32_t* __restrict__ row_model, int nm, const int* __restrict__ pact) {
  const int s = blockIdx.y;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = (int64_t)s * nm + row_model[r];
    if (!pact[p]) continue;
    double2 t = w[s * n + r];
    for (int i = 0; i < nv; ++i) {
      const double2 c = h[p * kMaxBasis + i], v = basis[s * sstride + (int64_t)i * vstride + r];
      t.x -= c.x * v.x - c.y * v.y;
      t.y -= c.x * v.y + c.y * v.x;
    }
    w[s * n + r] = t;
  }
}

// dst = src * scale_p (0 for the pairs that are done: their block of the basis is zero)
__global__ void k_vscale_seg(const double2* __restrict__ src, int64_t sstride_src, double2* __restrict__ dst,
                             int64_t sstride_dst, const double* __restrict__ scale, int64_t n,
                             const int32_t* __restrict__ row_model, int nm) {
  const int s = blockIdx.y;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const double a = scale[(int64_t)s * nm + row_model[r]];
    const double2 v = src[s * sstride_src + r];
    dst[s * sstride_dst + r] = make_double2(v.x * a, v.y * a);
  }
}

// t += sum_i y_{p,i} Z_i
__global__ void k_combo_seg(const double2* __restrict__ basis, int64_t sstride, int64_t vstride, int nv,
                            const double2* __restrict__ y, double2* __restrict__ t, int64_t n,
                            const int32_t* __restrict__ row_model, int nm, const int* __restrict__ pact) {
  const int s = blockIdx.y;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = (int64_t)s * nm + row_model[r];
    if (!pact[p]) continue;
    double ax = t[s * n + r].x, ay = t[s * n + r].y;
    for (int i = 0; i < nv; ++i) {
      const double2 c = y[p * kMaxBasis + i], v = basis[s * sstride + (int64_t)i * vstride + r];
      ax += c.x * v.x - c.y * v.y;
      ay += c.x * v.y + c.y * v.x;
    }
    t[s * n + r] = make_double2(ax, ay);
  }
}

// u = D z (front precision -> FP64), u of slot s at u + s * sstride
template <class V>
__global__ void k_unscale(const V* __restrict__ z, const double* __restrict__ dscale, int64_t n, double2* __restrict__ u,
                          int64_t sstride, const int* __restrict__ active) {
  const int s = blockIdx.y;
  if (!active[s]) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double d = dscale[s * n + i];
    V v = z[s * n + i];
    u[s * sstride + i] = make_double2(d * (double)v.x, d * (double)v.y);
  }
}

// ------------------------------------------------------------- host side
Workspace::~Workspace() {
  if (h_coef) cudaFreeHost(h_coef);
  if (h_norms) cudaFreeHost(h_norms);
  if (h_active) cudaFreeHost(h_active);
  if (h_stats) cudaFreeHost(h_stats);
  if (h_flag) cudaFreeHost(h_flag);
  if (h_mnorms) cudaFreeHost(h_mnorms);
  if (h_mdone) cudaFreeHost(h_mdone);
  if (h_ph) cudaFreeHost(h_ph);
  if (h_py) cudaFreeHost(h_py);
  if (h_pscal) cudaFreeHost(h_pscal);
  if (h_pact) cudaFreeHost(h_pact);
  if (h_h) cudaFreeHost(h_h);
  if (h_y) cudaFreeHost(h_y);
  if (h_scal) cudaFreeHost(h_scal);
  if (h_inner) cudaFreeHost(h_inner);
  for (int i = 0; i < 8; ++i)
    if (ev[i]) cudaEventDestroy(ev[i]);
  if (stream) cudaStreamDestroy(stream);
}

void make_coef(const Model& m, double w, Coef& c) {
  memset(&c, 0, sizeof(c));
  c.inv_w = 1.0 / w;
  c.fscale = 1.0;
  cplx c0 = group_coefficient(m.groups[0], w);
  c.a[CLS_STRUCT] = make_double2(c0.real(), c0.imag());
  c.b[CLS_STRUCT] = -w * w;
  c.a[CLS_FLUID] = make_double2(1.0 / (w * w), 0.0);
  c.b[CLS_FLUID] = -1.0;
  c.a[CLS_COUPLE] = make_double2(1.0, 0.0);
  c.b[CLS_COUPLE] = 0.0;
  for (size_t g = 1; g < m.groups.size() && g < (size_t)kMaxGroups; ++g) {
    cplx cg = group_coefficient(m.groups[g], w);
    c.g[g] = make_double2(cg.real(), cg.imag());
  }
}

int device_upload_symbolic(Model& m) {
  const Symbolic& S = *m.sym;
  if (!m.dsym) m.dsym.reset(new DeviceSymbolic());
  DeviceSymbolic& D = *m.dsym;
  const int T = (int)S.fronts.size();
  std::vector<int32_t> p(T), b(T), par(T), io(T), mo(T), co(T), po(T);
  std::vector<int64_t> off(T);
  std::vector<std::vector<int32_t>> kids(T);
  for (int t = 0; t < T; ++t) {
    const FrontInfo& F = S.fronts[t];
    p[t] = F.p; b[t] = F.b; par[t] = F.parent; io[t] = F.idx_off; mo[t] = F.map_off;
    co[t] = F.cb_off; po[t] = F.piv_off; off[t] = F.off;
    if (F.parent >= 0) kids[F.parent].push_back(t);
  }
  std::vector<int32_t> cptr(T + 1, 0), clist;
  for (int t = 0; t < T; ++t) {
    std::sort(kids[t].begin(), kids[t].end(), [&](int a, int c) { return S.fronts[a].child_slot < S.fronts[c].child_slot; });
    cptr[t + 1] = cptr[t] + (int32_t)kids[t].size();
    clist.insert(clist.end(), kids[t].begin(), kids[t].end());
  }
  ELP_CUDA(D.f_p.upload(p));
  ELP_CUDA(D.f_b.upload(b));
  ELP_CUDA(D.f_parent.upload(par));
  ELP_CUDA(D.f_idx_off.upload(io));
  ELP_CUDA(D.f_map_off.upload(mo));
  ELP_CUDA(D.f_cb_off.upload(co));
  ELP_CUDA(D.f_piv_off.upload(po));
  ELP_CUDA(D.f_off.upload(off));
  {
    std::vector<int64_t> fo(T), ff(T);
    for (int t = 0; t < T; ++t) {
      fo[t] = S.fronts[t].fac_off;
      ff[t] = S.fronts[t].off_full;
    }
    ELP_CUDA(D.f_fac.upload(fo));
    ELP_CUDA(D.f_off_full.upload(ff));
  }
  ELP_CUDA(D.scatter_order.upload(S.scatter_order));
  ELP_CUDA(D.entry_row.upload(S.entry_row));
  ELP_CUDA(D.front_dofs.upload(S.front_dofs));
  if (m.n_members > 1) {  // a front's DOFs all belong to one member (members share no node)
    std::vector<int32_t> fm(T, 0);
    for (int t = 0; t < T; ++t)
      if (S.fronts[t].p + S.fronts[t].b > 0) fm[t] = m.row_model[S.front_dofs[S.fronts[t].idx_off]];
    ELP_CUDA(D.f_member.upload(fm));
  }
  ELP_CUDA(D.parent_map.upload(S.parent_map));
  ELP_CUDA(D.child_ptr.upload(cptr));
  ELP_CUDA(D.child_list.upload(clist));
  ELP_CUDA(D.entry_local.upload(S.entry_local));
  ELP_CUDA(D.entry_owner.upload(S.entry_owner));
  std::vector<int32_t> ll, ea, nl;
  D.levels.assign(S.n_levels, DeviceSymbolic::Level());
  int maxc = std::max(1, S.max_children);
  for (int l = 0; l < S.n_levels; ++l) {
    auto& L = D.levels[l];
    L.start = (int)ll.size();
    L.count = (int)S.level_fronts[l].size();
    for (int t : S.level_fronts[l]) {
      ll.push_back(t);
      L.max_p = std::max(L.max_p, p[t]);
      L.max_b = std::max(L.max_b, b[t]);
      L.max_m = std::max(L.max_m, p[t] + b[t]);
      L.fac_max = std::max<int64_t>(L.fac_max, (int64_t)p[t] * p[t] + 2 * (int64_t)p[t] * b[t]);
    }
    L.new_start = (int)nl.size();
    L.new_count = (int)S.level_new[l].size();
    for (int t : S.level_new[l]) {
      nl.push_back(t);
      L.new_max_m2 = std::max<int64_t>(L.new_max_m2, (int64_t)(p[t] + b[t]) * (p[t] + b[t]));
    }
    L.ent_start = S.level_entry_start[l];
    L.ent_count = S.level_entry_start[l + 1] - S.level_entry_start[l];
    L.ea_start.assign(maxc, 0);
    L.ea_count.assign(maxc, 0);
    for (int k = 0; k < maxc; ++k) {
      L.ea_start[k] = (int)ea.size();
      for (int t : S.level_fronts[l])
        if (par[t] >= 0 && S.fronts[t].child_slot == k && b[t] > 0) {
          ea.push_back(t);
          L.ea_max_b = std::max(L.ea_max_b, b[t]);
        }
      L.ea_count[k] = (int)ea.size() - L.ea_start[k];
    }
  }
  // packed Schur operands (mixed path): per front with p, b > 0, tiles x chunks
  // blocks of A (L21, kSchurABlock bytes) then of B (U12, kSchurBBlock bytes)
  std::vector<int64_t> pbase(T, 0);
  for (int l = 0; l < S.n_levels; ++l) {
    auto& L = D.levels[l];
    int64_t off = 0;
    for (int t : S.level_fronts[l]) {
      pbase[t] = off;
      if (p[t] > 0 && b[t] > 0) {
        const int64_t tiles = (b[t] + kSchurTile - 1) / kSchurTile, nch = (p[t] + kTcKC - 1) / kTcKC;
        off += tiles * nch * (kSchurABlock + kSchurBBlock);
        L.pack_blocks = std::max<int>(L.pack_blocks, (int)(2 * tiles * nch));
        L.schur_tiles = std::max<int>(L.schur_tiles, (int)(tiles * tiles));
      }
    }
    L.pack_bytes = off;
  }
  D.pack_max = workspace_plan(m).pack_max;
  ELP_CUDA(D.pack_base.upload(pbase));
  ELP_CUDA(D.new_list.upload(nl));
  ELP_CUDA(D.level_list.upload(ll));
  ELP_CUDA(D.ea_list.upload(ea));
  D.n_fronts = T;
  D.arena = S.pool;
  D.arena_full = S.arena;
  D.fac = S.factor_stored;
  D.cb_total = S.cb_total;
  D.max_front = S.max_front;
  return ELP_OK;
}

// streaming multiprocessors of the current device (read once)
static int num_sms() {
  static const int v = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
  return v;
}

// Fronts per level / border rows that select packed Schur levels. Measured
// with the persistent packed kernel (32 frequencies per step, coupled 85k-DOF
// sweep): (36, 1024) 120.7, (80, 512) 121.1, (150, 300) 121.6 solves/s; with
// the vectorised pack pass (150, 300) 122.1, (300, 300) 123.2, (600, 200) 122.2.
int pack_max_count() {
  static const int v = [] {
    const char* e = getenv("ELP_PACK_COUNT");
    const int c = e ? atoi(e) : 300;
    return c < 0 ? 0 : c;
  }();
  return v;
}

int pack_min_border() {
  static const int v = [] {
    const char* e = getenv("ELP_PACK_MINB");
    const int c = e ? atoi(e) : 300;
    return c < 0 ? 0 : c;
  }();
  return v;
}

constexpr int kGmresRestart = 24;  // GMRES(24) of the mixed path

Tuning resolved_tuning(const Model& m) {
  static const int leaf_env = [] {
    const char* e = getenv("ELP_LEAF");
    const int v = e ? atoi(e) : 128;
    return v < 8 ? 8 : v;
  }();
  static const int lanes_env = [] {
    const char* e = getenv("ELP_LANES");
    int v = e ? atoi(e) : 4;
    return v < 1 ? 1 : v > 4 ? 4 : v;
  }();
  // 0 or negative: the default, except pack_count, where 0 means never
  Tuning t = m.tune;
  if (t.leaf <= 0) t.leaf = leaf_env;
  t.leaf = std::max(8, t.leaf);
  if (t.schur_tile != 32) t.schur_tile = 64;
  if (t.pack_count < 0) t.pack_count = pack_max_count();
  if (t.pack_minb <= 0) t.pack_minb = pack_min_border();
  if (t.lanes < 1) t.lanes = lanes_env;
  t.lanes = std::min(4, t.lanes);
  return t;
}

bool solve_global_forced() {
  static const bool v = getenv("ELP_SOLVE_GLOBAL") && std::string(getenv("ELP_SOLVE_GLOBAL")) == "1";
  return v;
}

WorkspacePlan workspace_plan(const Model& m) {
  const Symbolic& S = *m.sym;
  const Tuning tn = resolved_tuning(m);
  WorkspacePlan P;
  P.arena = S.pool;
  P.arena_full = S.arena;
  P.fac = S.factor_stored;
  P.cb_total = S.cb_total;
  static const bool pack_all_levels = getenv("ELP_TC_PACK") && std::string(getenv("ELP_TC_PACK")) == "all";
  for (int l = 0; l < S.n_levels; ++l) {
    DeviceSymbolic::Level L;
    L.count = (int)S.level_fronts[l].size();
    int64_t off = 0;
    for (int t : S.level_fronts[l]) {
      const FrontInfo& F = S.fronts[t];
      L.max_b = std::max(L.max_b, F.b);
      L.max_p = std::max(L.max_p, F.p);
      L.max_m = std::max(L.max_m, F.p + F.b);
      if (F.p > 0 && F.b > 0) {
        const int64_t tiles = (F.b + kSchurTile - 1) / kSchurTile, nch = (F.p + kTcKC - 1) / kTcKC;
        off += tiles * nch * (kSchurABlock + kSchurBBlock);
      }
    }
    P.max_count = std::max<int64_t>(P.max_count, L.count);
    if (pack_all_levels || packed_schur_level(L, tn)) P.pack_max = std::max(P.pack_max, off);
    for (int prec = 0; prec < 2; ++prec) {
      const int64_t elem = prec == ELP_MIXED ? sizeof(float2) : sizeof(double2);
      if (solve_level_global(L.max_m, L.max_p, elem))
        P.gvec[prec] = std::max<int64_t>(P.gvec[prec], (int64_t)L.count * (L.max_m + L.max_p));
    }
  }
  return P;
}

// Device bytes of the workspace `workspace_ensure` (+ the GMRES buffers of the
// mixed path) allocates for `slots` frequencies; the serving loop admits
// models against this figure, so it mirrors those allocations. Needs only the
// host symbolic phase (no device allocation has to happen first).
int64_t workspace_bytes(const Model& m, int precision, int slots, int store) {
  if (!m.sym) return 0;
  const WorkspacePlan D = workspace_plan(m);
  const int64_t n = m.n, S = slots;
  const int64_t elem = precision == ELP_MIXED ? sizeof(float2) : sizeof(double2);
  const int64_t nparts = std::min<int64_t>(1024, (n + 255) / 256);
  const int64_t max_count = D.max_count;
  const int64_t fronts = store == STORE_COMPACT ? D.arena + D.fac : D.arena_full;  // pool + factors, or whole fronts
  int64_t b = S * (fronts + std::max<int64_t>(1, D.cb_total) + 2 * n) * elem;          // fronts, cb, z, tb
  b += S * n * (4 + 8 + 3 * 16);                                               // perm, dscale, x, r, f
  b += S * (int64_t)(sizeof(Coef) * m.n_members + 16 + nparts * 16 + 4 + 32) + 4;  // coef, norms, partials, flags
  if (m.n_members > 1) b += S * m.n_members * 20;                                   // member norms, flags
  b += max_count * S * swapmap_ints<32>() * 4;
  b += S * D.gvec[precision == ELP_MIXED ? 1 : 0] * elem;                    // global solve vectors
  if (precision == ELP_MIXED) {
    b += S * D.pack_max;
    const int64_t rst = kGmresRestart;
    b += S * ((2 * rst + 2) * n * 16 + (int64_t)kMaxBasis * 16 * (4 + nparts) + 8 + 4);  // Vb, Zb, wv, Hessenberg
    if (m.n_members > 1) b += S * m.n_members * ((int64_t)kMaxBasis * 16 * 4 + 12);        // per-member GMRES
  }
  return b;
}

int64_t workspace_held(const Model& m, int precision) {
  int64_t b = 0;
  if (m.ws[precision]) b += workspace_bytes(m, precision, m.ws[precision]->slots, m.ws[precision]->store);
  for (const auto& w : m.ws_b[precision])
    if (w) b += workspace_bytes(m, precision, w->slots, w->store);
  return b;
}

static int workspace_alloc(Model& m, Workspace& w, int precision, int slots, int store);

int forced_store() {
  static const int v = [] {
    const char* e = getenv("ELP_FACTOR_STORE");
    if (e && std::string(e) == "full") return (int)STORE_FULL;
    if (e && std::string(e) == "compact") return (int)STORE_COMPACT;
    return -1;
  }();
  return v;
}

int choose_store(const Model& m, int precision, int slots, int64_t budget) {
  const int f = forced_store();
  if (f >= 0) return f;
  const int64_t full = workspace_bytes(m, precision, slots, STORE_FULL);
  // small trees: the pool holds most fronts at once and the compact store saves nothing
  if (full <= budget || workspace_bytes(m, precision, slots, STORE_COMPACT) >= full) return STORE_FULL;
  return STORE_COMPACT;
}

int workspace_ensure(Model& m, int precision, int slots, int lane, int store) {
  std::unique_ptr<Workspace>& W = lane ? m.ws_b[precision][lane - 1] : m.ws[precision];
  if (W && W->slots >= slots && W->store == store) return ELP_OK;
  W.reset();  // the old workspace goes before the new one is made
  // built aside and kept only when every allocation succeeded
  std::unique_ptr<Workspace> fresh(new Workspace());
  int rc = workspace_alloc(m, *fresh, precision, slots, store);
  if (rc) return rc;
  W = std::move(fresh);
  return ELP_OK;
}

static int workspace_alloc(Model& m, Workspace& w, int precision, int slots, int store) {
  w.precision = precision;
  w.slots = slots;
  w.store = store;
  w.elem = precision == ELP_MIXED ? sizeof(float2) : sizeof(double2);
  const DeviceSymbolic& D = *m.dsym;
  const int64_t n = m.n;
  w.arena_stride = store == STORE_COMPACT ? D.arena : D.arena_full;
  w.foff = store == STORE_COMPACT ? D.f_off.p : D.f_off_full.p;
  cudaError_t e = w.arena.alloc((size_t)slots * w.arena_stride * w.elem);
  if (e == cudaSuccess && store == STORE_COMPACT) e = w.fac.alloc((size_t)slots * D.fac * w.elem);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("front pool and factor store do not fit in device memory");
    return ELP_ERR_NOMEM;
  }
  ELP_CUDA(w.cb.alloc((size_t)slots * std::max<int64_t>(1, D.cb_total) * w.elem));
  ELP_CUDA(w.z.alloc((size_t)slots * n * w.elem));
  ELP_CUDA(w.tb.alloc((size_t)slots * n * w.elem));
  {
    const int64_t gv = workspace_plan(m).gvec[precision == ELP_MIXED ? 1 : 0];
    if (gv > 0) ELP_CUDA(w.gvec.alloc((size_t)slots * gv * w.elem));
  }
  ELP_CUDA(w.perm.alloc((size_t)slots * n));
  ELP_CUDA(w.dscale.alloc((size_t)slots * n));
  ELP_CUDA(w.x.alloc((size_t)slots * n));
  ELP_CUDA(w.r.alloc((size_t)slots * n));
  ELP_CUDA(w.f.alloc((size_t)slots * n));
  const int nm = m.n_members;
  ELP_CUDA(w.coef.alloc((size_t)slots * nm));
  if (nm > 1) {
    ELP_CUDA(w.mnorms.alloc((size_t)slots * nm * 2));
    ELP_CUDA(w.mdone.alloc((size_t)slots * nm));
  }
  ELP_CUDA(w.norms.alloc(2 * (size_t)slots));
  w.nparts = (int)std::min<int64_t>(1024, (n + 255) / 256);
  ELP_CUDA(w.partial.alloc((size_t)slots * w.nparts * 2));
  ELP_CUDA(w.active.alloc(slots));
  ELP_CUDA(w.stats.alloc(4 * (size_t)slots));
  {
    int max_count = 1;
    for (const auto& LV : D.levels) max_count = std::max(max_count, LV.count);
    ELP_CUDA(w.swapmap.alloc((size_t)max_count * slots * swapmap_ints<32>()));
  }
  ELP_CUDA(w.tc_err.alloc(1));
  ELP_CUDA(cudaMemset(w.tc_err.p, 0, sizeof(int)));
  if (precision == ELP_MIXED && D.pack_max > 0) ELP_CUDA(w.pack.alloc((size_t)slots * D.pack_max));
  ELP_CUDA(cudaMallocHost((void**)&w.h_coef, sizeof(Coef) * slots * nm));
  if (nm > 1) {
    ELP_CUDA(cudaMallocHost((void**)&w.h_mnorms, sizeof(double) * 2 * slots * nm));
    ELP_CUDA(cudaMallocHost((void**)&w.h_mdone, sizeof(int) * slots * nm));
  }
  ELP_CUDA(cudaMallocHost((void**)&w.h_norms, sizeof(double) * 2 * slots));
  ELP_CUDA(cudaMallocHost((void**)&w.h_active, sizeof(int) * slots));
  ELP_CUDA(cudaMallocHost((void**)&w.h_stats, sizeof(unsigned long long) * 4 * slots));
  ELP_CUDA(cudaMallocHost((void**)&w.h_flag, sizeof(int)));
  ELP_CUDA(cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking));
  for (int i = 0; i < 8; ++i) ELP_CUDA(cudaEventCreate(&w.ev[i]));
  return ELP_OK;
}

CombineArgs combine_args(const Model& m) {
  CombineArgs A;
  A.VK = m.dev->VK.p;
  A.VM = m.dev->VM.p;
  A.VKg = m.dev->VKg.p;
  A.cls = m.dev->cls.p;
  A.nnz = m.nnz;
  A.ngroups = (int)std::min<size_t>(m.groups.size(), kMaxGroups);
  A.row_model = m.n_members > 1 ? m.dev->row_model.p : nullptr;
  A.n_members = m.n_members;
  return A;
}

int numeric_system_values(Model& m, double omega, double2* out_dev) {
  DevBuf<Coef> c;
  Coef h;
  make_coef(m, omega, h);
  ELP_CUDA(c.upload(&h, 1));
  CombineArgs A = combine_args(m);
  PROF_LAUNCH(KC_VALUES, 0, k_values<<<1024, 256>>>(A, c.p, out_dev));
  ELP_CUDA(cudaGetLastError());
  ELP_CUDA(cudaDeviceSynchronize());
  return ELP_OK;
}

// dynamic shared-memory limits of the tensor-core kernels (once per process)
static int tc_kernel_attributes() {
  constexpr int NB = 32;
  static std::once_flag once;
  static cudaError_t e = cudaSuccess;
  std::call_once(once, [] {
    cudaError_t a = cudaFuncSetAttribute(k_gemm_tc<NB, 32, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kTcSmemBytes);
    cudaError_t b = cudaFuncSetAttribute(k_gemm_tc<NB, 32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kTcSmemBytes);
    cudaError_t c = cudaFuncSetAttribute(k_gemm_tc<NB, 64, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kTcSmemBytes);
    cudaError_t d = cudaFuncSetAttribute(k_schur_tc<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kSchurSmemBytes);
    e = a != cudaSuccess ? a : b != cudaSuccess ? b : c != cudaSuccess ? c : d;
  });
  ELP_CUDA(e);
  return ELP_OK;
}

template <class R>
static int factor_and_setup(Model& m, Workspace& w, int S_used, cudaStream_t st) {
  using V = typename Vec2<R>::T;
  constexpr int NB = sizeof(R) == 8 ? 32 : 32;
  DeviceSymbolic& D = *m.dsym;
  DeviceModel& G = *m.dev;
  const int64_t n = m.n;
  V* arena = reinterpret_cast<V*>(w.arena.p);
  CombineArgs A = combine_args(m);
  const Tuning tn = resolved_tuning(m);
  ELP_CUDA(cudaMemsetAsync(w.stats.p, 0, sizeof(unsigned long long) * 4 * S_used, st));
  {
    dim3 g((unsigned)std::min<int64_t>((n + 255) / 256, 4096), S_used);
    PROF_LAUNCH(KC_DSCALE, st, k_dscale<<<g, 256, 0, st>>>(A, w.coef.p, G.diag_idx.p, n, w.dscale.p));
  }
  V* fac = reinterpret_cast<V*>(w.fac.p);
  LevelArgs L;
  L.fp = D.f_p.p;
  L.fb = D.f_b.p;
  L.piv_off = D.f_piv_off.p;
  L.foff = w.foff;
  L.arena_size = w.arena_stride;
  L.n = n;
  L.fparent = D.f_parent.p;
  L.map_off = D.f_map_off.p;
  L.pmap = D.parent_map.p;
  L.fuse = 0;
  const R tiny = sizeof(R) == 8 ? (R)1e-10 : (R)1e-6;
  // FP32 fronts: Schur updates on the tensor cores (tcgen05, 3xTF32) unless ELP_TC=0
  static const bool use_tc = !(getenv("ELP_TC") && getenv("ELP_TC")[0] == '0');
  // Schur complement from packed operands (k_schur_tc) on the levels that gain from it;
  // ELP_TC_PACK=0 never, ELP_TC_PACK=all on every level (tests of small models)
  static const char* pack_env = getenv("ELP_TC_PACK");
  static const bool use_pack = !(pack_env && pack_env[0] == '0');
  static const bool pack_all = pack_env && std::string(pack_env) == "all";
  const bool tc = std::is_same<R, float>::value && use_tc;
  if (tc) {
    int rc = tc_kernel_attributes();
    if (rc) return rc;
  }
  const int panel_cap = kPanelSmemBytes / (NB * (int)sizeof(V));  // panel rows held in shared memory
  {
    static std::once_flag once;
    static cudaError_t e = cudaSuccess;
    std::call_once(once, [] {
      e = cudaFuncSetAttribute(k_panel<R, NB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kPanelSmemBytes);
    });
    ELP_CUDA(e);
  }
  // mode: GM_COL / GM_ROW / GM_SCHUR; rows_c, cols_c: upper bounds of the C block over the level
  auto gemm = [&](int mode, int k, int rows_c, int cols_c, const LevelArgs& L) {
    if (tc) {
      float2* fa = reinterpret_cast<float2*>(arena);
      if (mode == GM_SCHUR && tn.schur_tile == 32) {  // narrower tiles: more CTAs on short borders
        const int t = ((rows_c + 127) / 128) * ((cols_c + 31) / 32);
        dim3 g(L.count, S_used, (unsigned)std::min(65535, t));
        PROF_LAUNCH(KC_GEMM_TC, st, k_gemm_tc<NB, 32, false><<<g, kTcThreads, kTcSmemBytes, st>>>(L, fa, k, mode, w.tc_err.p));
      } else if (mode == GM_SCHUR) {
        const int t = ((rows_c + 127) / 128) * ((cols_c + 63) / 64);
        dim3 g(L.count, S_used, (unsigned)std::min(65535, t));
        PROF_LAUNCH(KC_GEMM_TC, st, k_gemm_tc<NB, 64, false><<<g, kTcThreads, kTcSmemBytes, st>>>(L, fa, k, mode, w.tc_err.p));
      } else if (mode == GM_COL) {
        dim3 g(L.count, S_used, (unsigned)std::min(65535, (rows_c + 127) / 128));
        PROF_LAUNCH(KC_GEMM_TC, st, k_gemm_tc<NB, 32, false><<<g, kTcThreads, kTcSmemBytes, st>>>(L, fa, k, mode, w.tc_err.p));
      } else {
        dim3 g(L.count, S_used, (unsigned)std::min(65535, (cols_c + 127) / 128));
        PROF_LAUNCH(KC_GEMM_TC, st, k_gemm_tc<NB, 32, true><<<g, kTcThreads, kTcSmemBytes, st>>>(L, fa, k, mode, w.tc_err.p));
      }
      return;
    }
    if (mode == GM_SCHUR) {
      const int t = ((rows_c + 63) / 64) * ((cols_c + 63) / 64);
      dim3 g(L.count, S_used, (unsigned)std::min(65535, t));
      PROF_LAUNCH(KC_GEMM, st, k_gemm<R, NB, 64, 64><<<g, 256, 0, st>>>(L, arena, k, mode));
    } else if (mode == GM_COL) {
      dim3 g(L.count, S_used, (unsigned)std::min(65535, (rows_c + 127) / 128));
      PROF_LAUNCH(KC_GEMM, st, k_gemm<R, NB, 128, 32><<<g, 256, 0, st>>>(L, arena, k, mode));
    } else {
      dim3 g(L.count, S_used, (unsigned)std::min(65535, (cols_c + 127) / 128));
      PROF_LAUNCH(KC_GEMM, st, k_gemm<R, NB, 32, 128><<<g, 256, 0, st>>>(L, arena, k, mode));
    }
  };
  for (size_t l = 0; l < D.levels.size(); ++l) {
    const auto& LV = D.levels[l];
    prof_set_level((int)l);
    if (LV.new_count > 0) {  // full fronts starting here: zeroed, then their entries of A(w) written
      dim3 gz(LV.new_count, S_used, (unsigned)std::min<int64_t>(65535, (LV.new_max_m2 + 4095) / 4096));
      PROF_LAUNCH(KC_SCATTER, st, k_zero_fronts<V><<<gz, 256, 0, st>>>(D.new_list.p + LV.new_start, D.f_p.p, D.f_b.p,
                                                                        w.foff, arena, w.arena_stride));
    }
    if (LV.ent_count > 0) {
      dim3 gs((unsigned)std::min<int64_t>((LV.ent_count + 255) / 256, 8192), S_used);
      PROF_LAUNCH(KC_SCATTER, st, k_scatter<V><<<gs, 256, 0, st>>>(A, w.coef.p, D.scatter_order.p + LV.ent_start,
                                                                    LV.ent_count, D.entry_row.p, G.col_idx.p,
                                                                    D.entry_owner.p, D.entry_local.p, w.foff,
                                                                    w.dscale.p, n, arena, w.arena_stride, w.stats.p));
    }
    L.list = D.level_list.p + LV.start;
    L.count = LV.count;
    const int steps = (LV.max_p + NB - 1) / NB;
    for (int k = 0; k < steps; ++k) {
      const int rows = LV.max_m - k * NB;       // rows k0..m-1 of the panel columns
      const int rest = LV.max_m - k * NB - 1;   // columns right of the panel (upper bound)
      if (k > 0) gemm(GM_COL, k, rows, NB, L);  // panel columns from all previous panels
      dim3 g1(LV.count, S_used);
      {
        const int rows_max = LV.max_p - k * NB;
        const size_t psm = (size_t)std::min(rows_max, panel_cap) * NB * sizeof(V);
        PROF_LAUNCH(KC_PANEL, st, k_panel<R, NB, true><<<g1, 256, psm, st>>>(L, arena, w.perm.p, k, tiny, w.stats.p,
                                                                            w.swapmap.p, panel_cap));
        if (rows_max > panel_cap)  // fronts whose panel rows exceed shared memory
          PROF_LAUNCH(KC_PANEL, st, k_panel<R, NB, false><<<g1, 256, 0, st>>>(L, arena, w.perm.p, k, tiny, w.stats.p,
                                                                             w.swapmap.p, panel_cap));
        dim3 gl(LV.count, S_used, (unsigned)std::min(65535, (LV.max_m + kLaswpCols - 1) / kLaswpCols));
        PROF_LAUNCH(KC_PANEL, st, k_laswp<R, NB><<<gl, 256, 0, st>>>(L, arena, w.swapmap.p, k));
      }
      if (LV.max_b > 0) {
        dim3 g2(LV.count, S_used, (unsigned)std::min(65535, (LV.max_b + 127) / 128));
        PROF_LAUNCH(KC_BORDER, st, k_border<R, NB><<<g2, 128, 0, st>>>(L, arena, k));
      }
      if (rest > 0) {
        if (k > 0) gemm(GM_ROW, k, NB, rest, L);  // pivot rows right of the panel from all previous panels
        dim3 g3(LV.count, S_used, (unsigned)std::min(65535, (rest + 127) / 128));
        g3.z = (unsigned)std::min(65535, (rest + urow_cols<R>() - 1) / urow_cols<R>());
        PROF_LAUNCH(KC_UROW, st, k_urow<R, NB><<<g3, 128, 0, st>>>(L, arena, k));
      }
    }
    if (LV.max_b > 0 && tc) {
      // Schur complement C -= L21 U12 added straight into each parent front (the
      // extend-add fused into the update's epilogue): one child slot per launch,
      // so no two fronts of a launch share a parent (fixed summation order)
      // few, large fronts (the top of the tree): operands split into TF32 planes once,
      // then bulk-copied by the MMA kernel (k_schur_tc); below, the converter kernel wins
      // (128-wide tiles waste work on short borders and the pack pass does not pay off)
      const bool packed = use_pack && w.pack.p && (pack_all || packed_schur_level(LV, tn));
      float2* fa = reinterpret_cast<float2*>(arena);
      uint32_t* pk = reinterpret_cast<uint32_t*>(w.pack.p);
      if (packed) {
        dim3 gp(LV.count, S_used, (unsigned)std::min(65535, LV.pack_blocks));
        PROF_LAUNCH(KC_PACK, st, k_pack_schur<NB><<<gp, 256, 0, st>>>(L, fa, pk, D.pack_base.p, LV.pack_bytes));
      }
      LevelArgs Lc = L;
      Lc.fuse = 1;
      for (size_t k = 0; k < LV.ea_count.size(); ++k) {
        if (!LV.ea_count[k]) continue;
        Lc.list = D.ea_list.p + LV.ea_start[k];
        Lc.count = LV.ea_count[k];
        if (packed) {
          // persistent CTAs (one per SM): about two waves over the launch, the
          // tiles of a front and slot split over gridDim.z of them
          const int64_t pairs = (int64_t)Lc.count * S_used;
          const int64_t gz = std::min<int64_t>(LV.schur_tiles, std::max<int64_t>(1, (2 * num_sms() + pairs - 1) / pairs));
          dim3 gs(Lc.count, S_used, (unsigned)gz);
          const int fault = fault_tc_wait() ? 1 : 0;  // host-side test switch (elp_fault_inject)
          PROF_LAUNCH(KC_SCHUR_TC, st, k_schur_tc<NB><<<gs, kSchurThreads, kSchurSmemBytes, st>>>(
                                          Lc, fa, pk, D.pack_base.p, LV.pack_bytes, w.tc_err.p, fault));
        } else {
          gemm(GM_SCHUR, 0, LV.ea_max_b, LV.ea_max_b, Lc);
        }
      }
    } else if (LV.max_b > 0) {
      gemm(GM_SCHUR, 0, LV.max_b, LV.max_b, L);  // Schur complement, depth p
    }
    if (!tc) {  // extend-add of the children's Schur complements into their parents
      for (size_t k = 0; k < LV.ea_count.size(); ++k) {
        if (!LV.ea_count[k]) continue;
        dim3 g5(LV.ea_count[k], S_used, (unsigned)std::min(65535, (LV.ea_max_b + 3) / 4));  // 4 columns per pass
        PROF_LAUNCH(KC_EXTEND_ADD, st, k_extend_add<R><<<g5, 256, 0, st>>>(D.ea_list.p + LV.ea_start[k], D.f_p.p, D.f_b.p,
                                                                           D.f_parent.p, D.f_map_off.p, w.foff,
                                                                           D.parent_map.p, arena, w.arena_stride));
      }
    }
    if (w.store == STORE_COMPACT) {  // the level's factors into the factor store; its full fronts are dead from here
      dim3 gc(LV.count, S_used, (unsigned)std::min<int64_t>(65535, (LV.fac_max + 2047) / 2048));
      PROF_LAUNCH(KC_SCATTER, st, k_compact<V><<<gc, 256, 0, st>>>(L.list, D.f_p.p, D.f_b.p, w.foff, D.f_fac.p,
                                                                    arena, w.arena_stride, fac, D.fac));
    }
  }
  prof_set_level(-1);
  ELP_CUDA(cudaGetLastError());
  return ELP_OK;
}

// threads of a pivot-block solve CTA: few for the many small fronts of the
// lower levels (more CTAs per SM), many for the few large fronts at the top
// (more rows of the trailing update in flight)
static int solve_threads(int max_p) { return max_p <= 128 ? 128 : max_p >= 512 ? 512 : 256; }

template <class R>
static int solve_sweep(Model& m, Workspace& w, int S_used, cudaStream_t st, const int* mask,
                       const int* pact = nullptr) {
  using V = typename Vec2<R>::T;
  DeviceSymbolic& D = *m.dsym;
  SolveArgs S;
  S.fp = D.f_p.p;
  S.fb = D.f_b.p;
  S.idx_off = D.f_idx_off.p;
  S.map_off = D.f_map_off.p;
  S.cb_off = D.f_cb_off.p;
  S.piv_off = D.f_piv_off.p;
  S.child_ptr = D.child_ptr.p;
  S.child_list = D.child_list.p;
  const bool compact = w.store == STORE_COMPACT;
  S.foff = compact ? D.f_fac.p : w.foff;  // the factor store (U12 with ld p), or the fronts in place
  S.u12_ld_p = compact ? 1 : 0;
  S.dofs = D.front_dofs.p;
  S.pmap = D.parent_map.p;
  S.arena_size = compact ? D.fac : w.arena_stride;
  S.n = m.n;
  S.cb_total = std::max<int64_t>(1, D.cb_total);
  S.active = mask;
  S.gvec = nullptr;
  S.gvec_stride = 0;
  S.fmember = D.f_member.p;
  S.pact = pact;
  S.nm = m.n_members;
  const V* arena = reinterpret_cast<const V*>(compact ? w.fac.p : w.arena.p);
  // levels whose front vector exceeds shared memory work on global slices
  auto level_buffers = [&](const DeviceSymbolic::Level& LV) -> bool {
    const bool glob = solve_level_global(LV.max_m, LV.max_p, sizeof(V));
    S.gvec = glob ? (void*)w.gvec.p : nullptr;
    S.gvec_stride = LV.max_m + LV.max_p;
    return glob;
  };
  V* z = reinterpret_cast<V*>(w.z.p);
  V* cb = reinterpret_cast<V*>(w.cb.p);
  for (size_t l = 0; l < D.levels.size(); ++l) {
    const auto& LV = D.levels[l];
    prof_set_level(32 + (int)l);  // solve sweeps: levels 32.. in the per-level table
    S.list = D.level_list.p + LV.start;
    S.count = LV.count;
    const bool glob = level_buffers(LV);
    if (glob && !w.gvec.p) { set_error("solve workspace lacks its global front vectors"); return ELP_ERR_STATE; }
    // front vector + permutation buffer
    size_t sm = glob ? 0 : (size_t)(LV.max_m + LV.max_p) * sizeof(V);
    auto fwd = glob ? k_forward<R, true> : k_forward<R, false>;
    PROF_LAUNCH(KC_FORWARD, st, fwd<<<dim3(LV.count, S_used), solve_threads(LV.max_p), sm, st>>>(S, arena, w.perm.p, z, cb));
    if (LV.max_b > 0) {
      const unsigned chunks = (unsigned)((LV.max_b + 31) / 32);
      auto fb = glob ? k_fwd_border<R, true> : k_fwd_border<R, false>;
      PROF_LAUNCH(KC_FWD_BORDER, st, fb<<<dim3(LV.count, S_used, chunks), 256, glob ? 0 : (size_t)LV.max_p * sizeof(V), st>>>(
                                      S, arena, z, cb));
    }
  }
  V* tb = reinterpret_cast<V*>(w.tb.p);
  for (int l = (int)D.levels.size() - 1; l >= 0; --l) {
    const auto& LV = D.levels[l];
    prof_set_level(32 + l);
    S.list = D.level_list.p + LV.start;
    S.count = LV.count;
    const bool glob = level_buffers(LV);
    if (glob && !w.gvec.p) { set_error("solve workspace lacks its global front vectors"); return ELP_ERR_STATE; }
    const unsigned chunks = (unsigned)((LV.max_p + 31) / 32);
    if (glob && LV.max_b > 0)
      PROF_LAUNCH(KC_BWD_U12, st, k_gather_border<R><<<dim3(LV.count, S_used), 256, 0, st>>>(S, z));
    auto bu = glob ? k_bwd_u12<R, true> : k_bwd_u12<R, false>;
    PROF_LAUNCH(KC_BWD_U12, st, bu<<<dim3(LV.count, S_used, chunks), 256,
                                     glob ? 0 : (size_t)std::max(1, LV.max_b) * sizeof(V), st>>>(S, arena, z, tb));
    size_t sm = glob ? 0 : (size_t)LV.max_p * sizeof(V);
    auto bwd = glob ? k_backward<R, true> : k_backward<R, false>;
    PROF_LAUNCH(KC_BACKWARD, st, bwd<<<dim3(LV.count, S_used), solve_threads(LV.max_p), sm, st>>>(S, arena, z, tb));
  }
  prof_set_level(-1);
  ELP_CUDA(cudaGetLastError());
  return ELP_OK;
}

template <class R>
static int solve_smem(const Model& m) {
  (void)m;  // levels beyond solve_smem_cap run on global slices (solve_sweep)
  // The limit is raised once per process to what the device allows: solves of
  // different models run concurrently (server workers), and a per-model value
  // set by one thread could lower the limit under another thread's launch.
  static std::once_flag once;
  static int rc = ELP_OK;
  std::call_once(once, [] {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (optin < kSolveSmemOptin) {
      rc = ELP_ERR_CUDA;
      return;
    }
    const void* fns[4] = {(const void*)k_forward<R, false>, (const void*)k_backward<R, false>,
                          (const void*)k_fwd_border<R, false>, (const void*)k_bwd_u12<R, false>};
    for (const void* fn : fns) {
      cudaFuncAttributes a;
      if (cudaFuncGetAttributes(&a, fn) != cudaSuccess ||
          optin - (int64_t)a.sharedSizeBytes < solve_smem_cap(sizeof(typename Vec2<R>::T)) ||
          cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)a.sharedSizeBytes) !=
              cudaSuccess) {
        cudaGetLastError();
        rc = ELP_ERR_CUDA;
      }
    }
  });
  if (rc) set_error("could not raise the shared-memory limit of the solve kernels");
  return rc;
}

// A group: each member's residual in the active slots; members at their
// tolerance (w.tol_member) have their residual rows zeroed. rel[s] becomes the
// norm of the rows still open relative to ||f|| of the slot, exactly 0 once
// every member is done.
static int group_mask(Model& m, Workspace& w, int S_used, cudaStream_t st, double* rel) {
  const int nm = m.n_members;
  const int64_t n = m.n;
  PROF_LAUNCH(KC_NORMS, st, k_member_norms<<<dim3(nm, S_used), 256, 0, st>>>(m.dev->member_off.p, nm, n, w.r.p,
                                                                                w.f.p, w.mnorms.p));
  ELP_CUDA(cudaMemcpyAsync(w.h_mnorms, w.mnorms.p, sizeof(double) * 2 * S_used * nm, cudaMemcpyDeviceToHost, st));
  ELP_CUDA(cudaStreamSynchronize(st));
  for (int s = 0; s < S_used; ++s) {
    double open = 0.0, ff = 0.0;
    for (int k = 0; k < nm; ++k) {
      const double rr = w.h_mnorms[2 * (s * nm + k)], fk = w.h_mnorms[2 * (s * nm + k) + 1];
      const double mrel = fk > 0 ? std::sqrt(rr / fk) : std::sqrt(rr);
      const int done = mrel <= w.tol_member ? 1 : 0;
      w.h_mdone[s * nm + k] = done;
      if (!done) open += rr;
      ff += fk;
    }
    if (w.h_active[s]) rel[s] = open == 0.0 ? 0.0 : (ff > 0 ? std::sqrt(open / ff) : std::sqrt(open));
  }
  ELP_CUDA(cudaMemcpyAsync(w.mdone.p, w.h_mdone, sizeof(int) * S_used * nm, cudaMemcpyHostToDevice, st));
  const dim3 g((unsigned)std::min<int64_t>((n + 255) / 256, 1024), S_used);
  PROF_LAUNCH(KC_KRYLOV, st, k_mask_members<<<g, 256, 0, st>>>(m.dev->row_model.p, w.mdone.p, nm, n, w.r.p,
                                                                w.active.p));
  return ELP_OK;
}

template <class R>
static int run_batch(Model& m, Workspace& w, int S_used, double tol, int max_iter, cudaStream_t st,
                     int* iters, float* ms) {
  using V = typename Vec2<R>::T;
  const int64_t n = m.n;
  DeviceModel& G = *m.dev;
  CombineArgs A = combine_args(m);
  int rc0 = solve_smem<R>(m);
  if (rc0) return rc0;
  for (int s = 0; s < S_used; ++s) { w.h_active[s] = 1; w.iters[s] = 0; }
  ELP_CUDA(cudaMemcpyAsync(w.active.p, w.h_active, sizeof(int) * S_used, cudaMemcpyHostToDevice, st));
  ELP_CUDA(cudaEventRecord(w.ev[0], st));
  int rc = factor_and_setup<R>(m, w, S_used, st);
  if (rc) return rc;
  ELP_CUDA(cudaEventRecord(w.ev[1], st));
  ELP_CUDA(cudaMemsetAsync(w.x.p, 0, sizeof(double2) * S_used * n, st));
  const dim3 gv((unsigned)std::min<int64_t>((n + 255) / 256, 4096), S_used);
  const dim3 gr((unsigned)w.nparts, S_used);
  int it = 0;
  float solve_ms = 0.f, refine_ms = 0.f;
  // initial residual r = f (x = 0)
  PROF_LAUNCH(KC_RESIDUAL, st, k_residual<<<gr, 256, 0, st>>>(A, w.coef.p, G.row_ptr.p, G.col_idx.p, n, w.x.p, w.f.p, w.r.p, w.partial.p,
                                 w.nparts, w.active.p, 1));
  for (it = 0; it < max_iter; ++it) {
    ELP_CUDA(cudaEventRecord(w.ev[2], st));
    PROF_LAUNCH(KC_RHS, st, k_rhs<V><<<gv, 256, 0, st>>>(A, w.coef.p, G.row_ptr.p, G.col_idx.p, w.r.p, n, w.dscale.p, n, reinterpret_cast<V*>(w.z.p), w.active.p));
    rc = solve_sweep<R>(m, w, S_used, st, w.active.p);
    if (rc) return rc;
    PROF_LAUNCH(KC_UPDATE, st, k_update<V><<<gv, 256, 0, st>>>(w.x.p, w.dscale.p, n, reinterpret_cast<const V*>(w.z.p), w.active.p));
    ELP_CUDA(cudaEventRecord(w.ev[3], st));
    PROF_LAUNCH(KC_RESIDUAL, st, k_residual<<<gr, 256, 0, st>>>(A, w.coef.p, G.row_ptr.p, G.col_idx.p, n, w.x.p, w.f.p, w.r.p, w.partial.p,
                                   w.nparts, w.active.p, 0));
    PROF_LAUNCH(KC_NORMS, st, k_norms<<<S_used, 256, 0, st>>>(w.partial.p, w.nparts, w.norms.p, w.active.p));
    ELP_CUDA(cudaMemcpyAsync(w.h_norms, w.norms.p, sizeof(double) * 2 * S_used, cudaMemcpyDeviceToHost, st));
    ELP_CUDA(cudaEventRecord(w.ev[4], st));
    ELP_CUDA(cudaEventSynchronize(w.ev[4]));
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, w.ev[2], w.ev[3]);
    cudaEventElapsedTime(&b, w.ev[3], w.ev[4]);
    solve_ms += a;
    refine_ms += b;
    bool all = true, changed = false;
    static const bool trace = getenv("ELP_TRACE") != nullptr;
    std::vector<double> grel(S_used, 0.0);
    if (m.n_members > 1) {  // a group: members at their tolerance stop changing
      rc = group_mask(m, w, S_used, st, grel.data());
      if (rc) return rc;
    }
    for (int s = 0; s < S_used; ++s) {
      if (!w.h_active[s]) continue;
      w.iters[s]++;
      double fn = w.h_norms[2 * s + 1];
      double rel = fn > 0 ? std::sqrt(w.h_norms[2 * s] / fn) : std::sqrt(w.h_norms[2 * s]);
      if (m.n_members > 1) rel = grel[s];
      if (trace) fprintf(stderr, "[elp] it %d slot %d rel_residual %.3e\n", it, s, rel);
      if (rel <= tol || !std::isfinite(rel)) { w.h_active[s] = 0; changed = true; }
      else all = false;
    }
    if (all) { ++it; break; }
    if (changed) ELP_CUDA(cudaMemcpyAsync(w.active.p, w.h_active, sizeof(int) * S_used, cudaMemcpyHostToDevice, st));
  }
  float fms = 0.f;
  cudaEventElapsedTime(&fms, w.ev[0], w.ev[1]);
  ms[0] = fms;
  ms[1] = solve_ms;
  ms[2] = refine_ms;
  *iters = it;
  return ELP_OK;
}

static int gmres_alloc(Workspace& w, int64_t n, int S, int rst, int nm = 1) {
  if (w.rst == rst) return ELP_OK;
  w.rst = 0;  // set once every buffer below exists, so a failed call is retried in full
  if (nm > 1) {  // a group: one Krylov process per (slot, member) pair
    const size_t P = (size_t)S * nm;
    ELP_CUDA(w.ph1.alloc(P * kMaxBasis));
    ELP_CUDA(w.ph2.alloc(P * kMaxBasis));
    ELP_CUDA(w.phn.alloc(P * kMaxBasis));
    ELP_CUDA(w.py.alloc(P * kMaxBasis));
    ELP_CUDA(w.pscal.alloc(P));
    ELP_CUDA(w.pact.alloc(P));
    if (!w.h_ph) ELP_CUDA(cudaMallocHost((void**)&w.h_ph, sizeof(double2) * 3 * P * kMaxBasis));
    if (!w.h_py) ELP_CUDA(cudaMallocHost((void**)&w.h_py, sizeof(double2) * P * kMaxBasis));
    if (!w.h_pscal) ELP_CUDA(cudaMallocHost((void**)&w.h_pscal, sizeof(double) * P));
    if (!w.h_pact) ELP_CUDA(cudaMallocHost((void**)&w.h_pact, sizeof(int) * P));
  }
  ELP_CUDA(w.Vb.alloc((size_t)S * (rst + 1) * n));
  ELP_CUDA(w.Zb.alloc((size_t)S * rst * n));
  ELP_CUDA(w.wv.alloc((size_t)S * n));
  ELP_CUDA(w.hd1.alloc((size_t)S * kMaxBasis));
  ELP_CUDA(w.hd2.alloc((size_t)S * kMaxBasis));
  ELP_CUDA(w.hnd.alloc((size_t)S * kMaxBasis));
  ELP_CUDA(w.ydev.alloc((size_t)S * kMaxBasis));
  ELP_CUDA(w.dpart.alloc((size_t)S * w.nparts * kMaxBasis));
  ELP_CUDA(w.scal.alloc(S));
  ELP_CUDA(w.inner.alloc(S));
  if (!w.h_h) ELP_CUDA(cudaMallocHost((void**)&w.h_h, sizeof(double2) * 3 * S * kMaxBasis));
  if (!w.h_y) ELP_CUDA(cudaMallocHost((void**)&w.h_y, sizeof(double2) * S * kMaxBasis));
  if (!w.h_scal) ELP_CUDA(cudaMallocHost((void**)&w.h_scal, sizeof(double) * S));
  if (!w.h_inner) ELP_CUDA(cudaMallocHost((void**)&w.h_inner, sizeof(int) * S));
  w.rst = rst;
  return ELP_OK;
}

// GMRES-IR: restarted right-preconditioned GMRES in FP64 with the
// front-precision factors as preconditioner (used for the mixed path, where
// plain refinement stalls once kappa(A) * eps_fp32 approaches 1).
template <class R>
static int run_gmres(Model& m, Workspace& w, int S_used, double tol, int max_cycles, cudaStream_t st, float* ms) {
  using V = typename Vec2<R>::T;
  typedef std::complex<double> cd;
  const int64_t n = m.n;
  DeviceModel& G = *m.dev;
  CombineArgs A = combine_args(m);
  int rc0 = solve_smem<R>(m);
  if (rc0) return rc0;
  const int RST = kGmresRestart;
  int rc = gmres_alloc(w, n, w.slots, RST);
  if (rc) return rc;
  const int64_t vst = (int64_t)(RST + 1) * n;  // slot stride of the Arnoldi basis V
  const int64_t zst = (int64_t)RST * n;        // slot stride of Z = M^-1 V
  for (int s = 0; s < S_used; ++s) { w.h_active[s] = 1; w.iters[s] = 0; }
  ELP_CUDA(cudaMemcpyAsync(w.active.p, w.h_active, sizeof(int) * S_used, cudaMemcpyHostToDevice, st));
  ELP_CUDA(cudaEventRecord(w.ev[0], st));
  rc = factor_and_setup<R>(m, w, S_used, st);
  if (rc) return rc;
  ELP_CUDA(cudaEventRecord(w.ev[1], st));
  ELP_CUDA(cudaMemsetAsync(w.x.p, 0, sizeof(double2) * S_used * n, st));
  const dim3 gv((unsigned)std::min<int64_t>((n + 255) / 256, 4096), S_used);
  const dim3 gr((unsigned)w.nparts, S_used);
  V* z = reinterpret_cast<V*>(w.z.p);
  // dot products: few blocks per slot, so each thread sums several entries before
  // the (FP64, costly) block reduction of every basis vector
  const int nd = std::min(w.nparts, 64);
  const dim3 gd((unsigned)nd, S_used);
  static const bool trace = getenv("ELP_TRACE") != nullptr;
  std::vector<double> fn(S_used), rel(S_used);
  auto residual = [&](int x_zero) -> int {
    PROF_LAUNCH(KC_RESIDUAL, st, k_residual<<<gr, 256, 0, st>>>(A, w.coef.p, G.row_ptr.p, G.col_idx.p, n, w.x.p, w.f.p,
                                                                   w.r.p, w.partial.p, w.nparts, w.active.p, x_zero));
    PROF_LAUNCH(KC_NORMS, st, k_norms<<<S_used, 256, 0, st>>>(w.partial.p, w.nparts, w.norms.p, w.active.p));
    ELP_CUDA(cudaMemcpyAsync(w.h_norms, w.norms.p, sizeof(double) * 2 * S_used, cudaMemcpyDeviceToHost, st));
    ELP_CUDA(cudaStreamSynchronize(st));
    for (int s = 0; s < S_used; ++s) {
      if (!w.h_active[s]) continue;
      fn[s] = std::sqrt(w.h_norms[2 * s + 1]);
      rel[s] = fn[s] > 0 ? std::sqrt(w.h_norms[2 * s]) / fn[s] : std::sqrt(w.h_norms[2 * s]);
    }
    // a group: members at their tolerance stop changing; rel is the open rows' residual
    if (m.n_members > 1) return group_mask(m, w, S_used, st, rel.data());
    return ELP_OK;
  };
  auto precond = [&](const double2* src, int64_t sstride, const int* mask) -> int {
    PROF_LAUNCH(KC_RHS, st, k_rhs<V><<<gv, 256, 0, st>>>(A, w.coef.p, G.row_ptr.p, G.col_idx.p, src, sstride, w.dscale.p, n, z, mask));
    return solve_sweep<R>(m, w, S_used, st, mask);
  };
  // a tensor-core wait that ran out left the factors incomplete: stop before
  // the Krylov cycles (the flag is read back with the first residual's sync)
  ELP_CUDA(cudaMemcpyAsync(w.h_flag, w.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  rc = residual(1);  // x = 0
  if (rc) return rc;
  if (*w.h_flag) {
    set_error("a tensor-core Schur update gave up waiting for its MMAs");
    return ELP_ERR_CUDA;
  }
  std::vector<std::vector<cd>> H(S_used, std::vector<cd>((RST + 1) * RST));
  std::vector<std::vector<cd>> g(S_used, std::vector<cd>(RST + 1)), sn(S_used, std::vector<cd>(RST));
  std::vector<std::vector<double>> cs(S_used, std::vector<double>(RST));
  std::vector<int> ncol(S_used);
  float solve_ms = 0.f;
  for (int cycle = 0; cycle < max_cycles; ++cycle) {
    bool any = false;
    for (int s = 0; s < S_used; ++s) {
      if (w.h_active[s] && (rel[s] <= tol || !std::isfinite(rel[s]))) w.h_active[s] = 0;
      any |= w.h_active[s] != 0;
      w.h_inner[s] = w.h_active[s];
      w.h_scal[s] = w.h_active[s] ? 1.0 / (rel[s] * fn[s]) : 0.0;
      ncol[s] = 0;
      if (w.h_active[s]) {
        std::fill(g[s].begin(), g[s].end(), cd(0));
        g[s][0] = rel[s] * fn[s];
      }
      if (trace && w.h_active[s]) fprintf(stderr, "[elp] gmres cycle %d slot %d rel_residual %.3e\n", cycle, s, rel[s]);
    }
    if (!any) break;
    ELP_CUDA(cudaMemcpyAsync(w.active.p, w.h_active, sizeof(int) * S_used, cudaMemcpyHostToDevice, st));
    ELP_CUDA(cudaMemcpyAsync(w.inner.p, w.h_inner, sizeof(int) * S_used, cudaMemcpyHostToDevice, st));
    ELP_CUDA(cudaMemcpyAsync(w.scal.p, w.h_scal, sizeof(double) * S_used, cudaMemcpyHostToDevice, st));
    PROF_LAUNCH(KC_KRYLOV, st, k_vscale<<<gv, 256, 0, st>>>(w.r.p, w.Vb.p, vst, w.scal.p, n, w.inner.p));
    for (int j = 0; j < RST; ++j) {
      ELP_CUDA(cudaEventRecord(w.ev[2], st));
      rc = precond(w.Vb.p + (int64_t)j * n, vst, w.inner.p);
      if (rc) return rc;
      ELP_CUDA(cudaEventRecord(w.ev[3], st));
      // Z_j = M^-1 V_j kept in FP64 (flexible GMRES: the update uses Z y, so
      // rounding of the front-precision solve never enters the Arnoldi relation)
      PROF_LAUNCH(KC_KRYLOV, st, k_unscale<V><<<gv, 256, 0, st>>>(z, w.dscale.p, n, w.Zb.p + (int64_t)j * n, zst, w.inner.p));
      PROF_LAUNCH(KC_SPMV, st, k_spmv<<<gr, 256, 0, st>>>(A, w.coef.p, G.row_ptr.p, G.col_idx.p, n,
                                                                 w.Zb.p + (int64_t)j * n, zst, w.wv.p, w.inner.p));
      const int nv = j + 1;
      PROF_LAUNCH(KC_KRYLOV, st, k_dots<<<gd, 256, 0, st>>>(w.Vb.p, vst, n, nv, w.wv.p, n, w.dpart.p, nd, w.inner.p));
      PROF_LAUNCH(KC_KRYLOV, st, k_dots_reduce<<<S_used, 32, 0, st>>>(w.dpart.p, nd, nv, w.hd1.p, w.inner.p));
      PROF_LAUNCH(KC_KRYLOV, st, k_gs<<<gv, 256, 0, st>>>(w.Vb.p, vst, n, nv, w.hd1.p, w.wv.p, n, w.inner.p));
      PROF_LAUNCH(KC_KRYLOV, st, k_dots<<<gd, 256, 0, st>>>(w.Vb.p, vst, n, nv, w.wv.p, n, w.dpart.p, nd, w.inner.p));
      PROF_LAUNCH(KC_KRYLOV, st, k_dots_reduce<<<S_used, 32, 0, st>>>(w.dpart.p, nd, nv, w.hd2.p, w.inner.p));
      PROF_LAUNCH(KC_KRYLOV, st, k_gs<<<gv, 256, 0, st>>>(w.Vb.p, vst, n, nv, w.hd2.p, w.wv.p, n, w.inner.p));
      PROF_LAUNCH(KC_KRYLOV, st, k_dots<<<gd, 256, 0, st>>>(w.wv.p, n, 0, 1, w.wv.p, n, w.dpart.p, nd, w.inner.p));
      PROF_LAUNCH(KC_KRYLOV, st, k_dots_reduce<<<S_used, 32, 0, st>>>(w.dpart.p, nd, 1, w.hnd.p, w.inner.p));
      ELP_CUDA(cudaMemcpyAsync(w.h_h, w.hd1.p, sizeof(double2) * S_used * kMaxBasis, cudaMemcpyDeviceToHost, st));
      ELP_CUDA(cudaMemcpyAsync(w.h_h + S_used * kMaxBasis, w.hd2.p, sizeof(double2) * S_used * kMaxBasis,
                               cudaMemcpyDeviceToHost, st));
      ELP_CUDA(cudaMemcpyAsync(w.h_h + 2 * S_used * kMaxBasis, w.hnd.p, sizeof(double2) * S_used * kMaxBasis,
                               cudaMemcpyDeviceToHost, st));
      ELP_CUDA(cudaStreamSynchronize(st));
      float a = 0.f;
      cudaEventElapsedTime(&a, w.ev[2], w.ev[3]);
      solve_ms += a;
      bool more = false;
      for (int s = 0; s < S_used; ++s) {
        if (!w.h_inner[s]) continue;
        w.iters[s]++;
        cd* Hs = H[s].data();  // column-major (RST + 1) x RST
        for (int i = 0; i <= j; ++i) {
          double2 h1 = w.h_h[s * kMaxBasis + i], h2 = w.h_h[(S_used + s) * kMaxBasis + i];
          Hs[j * (RST + 1) + i] = cd(h1.x + h2.x, h1.y + h2.y);
        }
        const double hn = std::sqrt(std::max(0.0, w.h_h[(2 * S_used + s) * kMaxBasis].x));
        Hs[j * (RST + 1) + j + 1] = cd(hn, 0.0);
        for (int i = 0; i < j; ++i) {  // previous rotations
          cd a0 = Hs[j * (RST + 1) + i], b0 = Hs[j * (RST + 1) + i + 1];
          Hs[j * (RST + 1) + i] = cs[s][i] * a0 + sn[s][i] * b0;
          Hs[j * (RST + 1) + i + 1] = -std::conj(sn[s][i]) * a0 + cs[s][i] * b0;
        }
        cd a0 = Hs[j * (RST + 1) + j], b0 = Hs[j * (RST + 1) + j + 1];
        double rho = std::sqrt(std::norm(a0) + std::norm(b0));
        if (std::abs(a0) == 0.0) { cs[s][j] = 0.0; sn[s][j] = cd(1.0, 0.0); }
        else {
          cs[s][j] = std::abs(a0) / rho;
          sn[s][j] = (a0 / std::abs(a0)) * std::conj(b0) / rho;
        }
        Hs[j * (RST + 1) + j] = cs[s][j] * a0 + sn[s][j] * b0;
        Hs[j * (RST + 1) + j + 1] = 0.0;
        g[s][j + 1] = -std::conj(sn[s][j]) * g[s][j];
        g[s][j] = cs[s][j] * g[s][j];
        ncol[s] = j + 1;
        const double est = std::abs(g[s][j + 1]) / fn[s];
        if (trace) fprintf(stderr, "[elp]   arnoldi %d slot %d estimate %.3e\n", j, s, est);
        if (est <= 0.5 * tol || hn <= 1e-300 || j == RST - 1 || !std::isfinite(est)) w.h_inner[s] = 0;
        else more = true;
        w.h_scal[s] = hn > 0 ? 1.0 / hn : 0.0;
      }
      ELP_CUDA(cudaMemcpyAsync(w.scal.p, w.h_scal, sizeof(double) * S_used, cudaMemcpyHostToDevice, st));
      PROF_LAUNCH(KC_KRYLOV, st, k_vscale<<<gv, 256, 0, st>>>(w.wv.p, w.Vb.p + (int64_t)(j + 1) * n, vst, w.scal.p, n, w.inner.p));
      ELP_CUDA(cudaMemcpyAsync(w.inner.p, w.h_inner, sizeof(int) * S_used, cudaMemcpyHostToDevice, st));
      if (!more) break;
    }
    // x += M^-1 V y
    int nvmax = 0;
    for (int s = 0; s < S_used; ++s) {
      for (int i = 0; i < kMaxBasis; ++i) w.h_y[s * kMaxBasis + i] = make_double2(0, 0);
      if (!w.h_active[s]) continue;
      const int k = ncol[s];
      nvmax = std::max(nvmax, k);
      std::vector<cd> y(k);
      const cd* Hs = H[s].data();
      for (int i = k - 1; i >= 0; --i) {
        cd t = g[s][i];
        for (int c = i + 1; c < k; ++c) t -= Hs[c * (RST + 1) + i] * y[c];
        y[i] = t / Hs[i * (RST + 1) + i];
      }
      for (int i = 0; i < k; ++i) w.h_y[s * kMaxBasis + i] = make_double2(y[i].real(), y[i].imag());
    }
    ELP_CUDA(cudaMemcpyAsync(w.ydev.p, w.h_y, sizeof(double2) * S_used * kMaxBasis, cudaMemcpyHostToDevice, st));
    PROF_LAUNCH(KC_UPDATE, st, k_combo<<<gv, 256, 0, st>>>(w.Zb.p, zst, n, nvmax, w.ydev.p, w.x.p, n, w.active.p));
    rc = residual(0);
    if (rc) return rc;
  }
  ELP_CUDA(cudaGetLastError());
  float fms = 0.f;
  cudaEventElapsedTime(&fms, w.ev[0], w.ev[1]);
  ms[0] = fms;
  ms[1] = solve_ms;
  ms[2] = 0.f;
  return ELP_OK;
}

// GMRES-IR for a group: the factorisation and the preconditioner sweeps run
// over the whole group (one launch per tree level for all members), but each
// (slot, member) pair p = s * nm + k has its own Krylov process -- its own dot
// products over its rows, Hessenberg matrix, rotations and update -- exactly
// the process the member would run alone, with its own stopping test
// ||r_k|| / ||f_k|| <= tol. A and the preconditioner are block diagonal, so
// the pairs only share launches: a member whose frequency is hard (or that sits
// at its FP64 floor) slows and fails no other member.
template <class R>
static int run_gmres_group(Model& m, Workspace& w, int S_used, double tol, int max_cycles, cudaStream_t st, float* ms) {
  using V = typename Vec2<R>::T;
  typedef std::complex<double> cd;
  const int64_t n = m.n;
  const int nm = m.n_members;
  const int64_t P = (int64_t)S_used * nm;
  DeviceModel& G = *m.dev;
  CombineArgs A = combine_args(m);
  int rc = solve_smem<R>(m);
  if (rc) return rc;
  const int RST = kGmresRestart;
  rc = gmres_alloc(w, n, w.slots, RST, nm);
  if (rc) return rc;
  const int64_t vst = (int64_t)(RST + 1) * n, zst = (int64_t)RST * n;
  for (int s = 0; s < S_used; ++s) { w.h_active[s] = 1; w.iters[s] = 0; }
  ELP_CUDA(cudaMemcpyAsync(w.active.p, w.h_active, sizeof(int) * S_used, cudaMemcpyHostToDevice, st));
  ELP_CUDA(cudaEventRecord(w.ev[0], st));
  rc = factor_and_setup<R>(m, w, S_used, st);
  if (rc) return rc;
  ELP_CUDA(cudaEventRecord(w.ev[1], st));
  ELP_CUDA(cudaMemsetAsync(w.x.p, 0, sizeof(double2) * S_used * n, st));
  const dim3 gv((unsigned)std::min<int64_t>((n + 255) / 256, 4096), S_used);
  const dim3 gr((unsigned)w.nparts, S_used);
  const dim3 gp((unsigned)nm, S_used);
  V* z = reinterpret_cast<V*>(w.z.p);
  const int64_t* off = G.member_off.p;
  const int32_t* rmod = G.row_model.p;
  std::vector<double> fn(P), rel(P);
  // masked: only the rows of the pairs in w.pact (those whose x changed this
  // cycle) are recomputed; the others keep their residual rows
  auto residual = [&](int x_zero, bool masked) -> int {
    CombineArgs Ar = A;
    if (masked) Ar.pact = w.pact.p;
    PROF_LAUNCH(KC_RESIDUAL, st, k_residual<<<gr, 256, 0, st>>>(Ar, w.coef.p, G.row_ptr.p, G.col_idx.p, n, w.x.p, w.f.p,
                                                                   w.r.p, w.partial.p, w.nparts, w.active.p, x_zero));
    PROF_LAUNCH(KC_NORMS, st, k_member_norms<<<gp, 256, 0, st>>>(off, nm, n, w.r.p, w.f.p, w.mnorms.p));
    ELP_CUDA(cudaMemcpyAsync(w.h_mnorms, w.mnorms.p, sizeof(double) * 2 * P, cudaMemcpyDeviceToHost, st));
    ELP_CUDA(cudaStreamSynchronize(st));
    for (int64_t q = 0; q < P; ++q) {
      const double rr = w.h_mnorms[2 * q], ff = w.h_mnorms[2 * q + 1];
      fn[q] = std::sqrt(ff);
      rel[q] = ff > 0 ? std::sqrt(rr / ff) : std::sqrt(rr);
    }
    return ELP_OK;
  };
  // the pairs that are done have zero rows in every later basis vector (the basis scale of
  // their block is 0); the products and the preconditioner skip their rows and fronts, and
  // the kernels that read those rows (segmented dots, Gram-Schmidt, combination) skip them
  // too, so what the skipped rows hold never reaches an open pair. The buffers start zeroed.
  CombineArgs Am = A;
  Am.pact = w.pact.p;
  ELP_CUDA(cudaMemsetAsync(w.Vb.p, 0, sizeof(double2) * (size_t)w.slots * (RST + 1) * n, st));
  ELP_CUDA(cudaMemsetAsync(w.Zb.p, 0, sizeof(double2) * (size_t)w.slots * RST * n, st));
  ELP_CUDA(cudaMemsetAsync(w.wv.p, 0, sizeof(double2) * (size_t)w.slots * n, st));
  ELP_CUDA(cudaMemsetAsync(w.z.p, 0, w.elem * (size_t)w.slots * n, st));
  auto precond = [&](const double2* src, int64_t sstride, const int* mask) -> int {
    PROF_LAUNCH(KC_RHS, st, k_rhs<V><<<gv, 256, 0, st>>>(Am, w.coef.p, G.row_ptr.p, G.col_idx.p, src, sstride, w.dscale.p, n, z, mask));
    return solve_sweep<R>(m, w, S_used, st, mask, w.pact.p);
  };
  // a tensor-core wait that ran out left the factors incomplete (read with the first residual)
  ELP_CUDA(cudaMemcpyAsync(w.h_flag, w.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  rc = residual(1, false);
  if (rc) return rc;
  if (*w.h_flag) {
    set_error("a tensor-core Schur update gave up waiting for its MMAs");
    return ELP_ERR_CUDA;
  }
  std::vector<std::vector<cd>> H(P, std::vector<cd>((RST + 1) * RST)), g(P, std::vector<cd>(RST + 1)),
      sn(P, std::vector<cd>(RST));
  std::vector<std::vector<double>> cs(P, std::vector<double>(RST));
  std::vector<int> ncol(P), open(P);
  float solve_ms = 0.f;
  auto upload_pairs = [&]() -> int {
    ELP_CUDA(cudaMemcpyAsync(w.pact.p, w.h_pact, sizeof(int) * P, cudaMemcpyHostToDevice, st));
    ELP_CUDA(cudaMemcpyAsync(w.pscal.p, w.h_pscal, sizeof(double) * P, cudaMemcpyHostToDevice, st));
    ELP_CUDA(cudaMemcpyAsync(w.inner.p, w.h_inner, sizeof(int) * S_used, cudaMemcpyHostToDevice, st));
    return ELP_OK;
  };
  for (int cycle = 0; cycle < max_cycles; ++cycle) {
    bool any = false;
    for (int s = 0; s < S_used; ++s) w.h_inner[s] = 0;
    for (int64_t q = 0; q < P; ++q) {
      open[q] = rel[q] > tol && std::isfinite(rel[q]);
      w.h_pact[q] = open[q];
      w.h_pscal[q] = open[q] ? 1.0 / (rel[q] * fn[q]) : 0.0;
      ncol[q] = 0;
      if (open[q]) {
        std::fill(g[q].begin(), g[q].end(), cd(0));
        g[q][0] = rel[q] * fn[q];
        w.h_inner[q / nm] = 1;
        any = true;
      }
    }
    if (!any) break;
    for (int s = 0; s < S_used; ++s) w.h_active[s] = w.h_inner[s];
    ELP_CUDA(cudaMemcpyAsync(w.active.p, w.h_active, sizeof(int) * S_used, cudaMemcpyHostToDevice, st));
    rc = upload_pairs();
    if (rc) return rc;
    PROF_LAUNCH(KC_KRYLOV, st, k_vscale_seg<<<gv, 256, 0, st>>>(w.r.p, n, w.Vb.p, vst, w.pscal.p, n, rmod, nm));
    for (int j = 0; j < RST; ++j) {
      ELP_CUDA(cudaEventRecord(w.ev[2], st));
      rc = precond(w.Vb.p + (int64_t)j * n, vst, w.inner.p);
      if (rc) return rc;
      ELP_CUDA(cudaEventRecord(w.ev[3], st));
      PROF_LAUNCH(KC_KRYLOV, st, k_unscale<V><<<gv, 256, 0, st>>>(z, w.dscale.p, n, w.Zb.p + (int64_t)j * n, zst, w.inner.p));
      PROF_LAUNCH(KC_SPMV, st, k_spmv<<<gr, 256, 0, st>>>(Am, w.coef.p, G.row_ptr.p, G.col_idx.p, n,
                                                                 w.Zb.p + (int64_t)j * n, zst, w.wv.p, w.inner.p));
      const int nv = j + 1;
      PROF_LAUNCH(KC_KRYLOV, st, k_dots_seg<<<gp, 256, 0, st>>>(w.Vb.p, vst, n, nv, w.wv.p, n, off, nm, w.ph1.p, w.pact.p));
      PROF_LAUNCH(KC_KRYLOV, st, k_gs_seg<<<gv, 256, 0, st>>>(w.Vb.p, vst, n, nv, w.ph1.p, w.wv.p, n, rmod, nm, w.pact.p));
      PROF_LAUNCH(KC_KRYLOV, st, k_dots_seg<<<gp, 256, 0, st>>>(w.Vb.p, vst, n, nv, w.wv.p, n, off, nm, w.ph2.p, w.pact.p));
      PROF_LAUNCH(KC_KRYLOV, st, k_gs_seg<<<gv, 256, 0, st>>>(w.Vb.p, vst, n, nv, w.ph2.p, w.wv.p, n, rmod, nm, w.pact.p));
      PROF_LAUNCH(KC_KRYLOV, st, k_dots_seg<<<gp, 256, 0, st>>>(w.wv.p, n, 0, 1, w.wv.p, n, off, nm, w.phn.p, w.pact.p));
      ELP_CUDA(cudaMemcpyAsync(w.h_ph, w.ph1.p, sizeof(double2) * P * kMaxBasis, cudaMemcpyDeviceToHost, st));
      ELP_CUDA(cudaMemcpyAsync(w.h_ph + P * kMaxBasis, w.ph2.p, sizeof(double2) * P * kMaxBasis,
                               cudaMemcpyDeviceToHost, st));
      ELP_CUDA(cudaMemcpyAsync(w.h_ph + 2 * P * kMaxBasis, w.phn.p, sizeof(double2) * P * kMaxBasis,
                               cudaMemcpyDeviceToHost, st));
      ELP_CUDA(cudaStreamSynchronize(st));
      float a = 0.f;
      cudaEventElapsedTime(&a, w.ev[2], w.ev[3]);
      solve_ms += a;
      for (int s = 0; s < S_used; ++s)
        if (w.h_inner[s]) w.iters[s]++;
      bool more = false;
      for (int s = 0; s < S_used; ++s) w.h_inner[s] = 0;
      for (int64_t q = 0; q < P; ++q) {
        if (!w.h_pact[q]) { w.h_pscal[q] = 0.0; continue; }
        cd* Hs = H[q].data();  // column-major (RST + 1) x RST
        for (int i = 0; i <= j; ++i) {
          const double2 h1 = w.h_ph[q * kMaxBasis + i], h2 = w.h_ph[(P + q) * kMaxBasis + i];
          Hs[j * (RST + 1) + i] = cd(h1.x + h2.x, h1.y + h2.y);
        }
        const double hn = std::sqrt(std::max(0.0, w.h_ph[(2 * P + q) * kMaxBasis].x));
        Hs[j * (RST + 1) + j + 1] = cd(hn, 0.0);
        for (int i = 0; i < j; ++i) {  // previous rotations
          const cd a0 = Hs[j * (RST + 1) + i], b0 = Hs[j * (RST + 1) + i + 1];
          Hs[j * (RST + 1) + i] = cs[q][i] * a0 + sn[q][i] * b0;
          Hs[j * (RST + 1) + i + 1] = -std::conj(sn[q][i]) * a0 + cs[q][i] * b0;
        }
        const cd a0 = Hs[j * (RST + 1) + j], b0 = Hs[j * (RST + 1) + j + 1];
        const double rho = std::sqrt(std::norm(a0) + std::norm(b0));
        if (std::abs(a0) == 0.0) { cs[q][j] = 0.0; sn[q][j] = cd(1.0, 0.0); }
        else {
          cs[q][j] = std::abs(a0) / rho;
          sn[q][j] = (a0 / std::abs(a0)) * std::conj(b0) / rho;
        }
        Hs[j * (RST + 1) + j] = cs[q][j] * a0 + sn[q][j] * b0;
        Hs[j * (RST + 1) + j + 1] = 0.0;
        g[q][j + 1] = -std::conj(sn[q][j]) * g[q][j];
        g[q][j] = cs[q][j] * g[q][j];
        ncol[q] = j + 1;
        const double est = std::abs(g[q][j + 1]) / fn[q];
        if (est <= 0.5 * tol || hn <= 1e-300 || j == RST - 1 || !std::isfinite(est)) {
          w.h_pact[q] = 0;
          w.h_pscal[q] = 0.0;
        } else {
          more = true;
          w.h_inner[q / nm] = 1;
          w.h_pscal[q] = hn > 0 ? 1.0 / hn : 0.0;
        }
      }
      rc = upload_pairs();
      if (rc) return rc;
      PROF_LAUNCH(KC_KRYLOV, st, k_vscale_seg<<<gv, 256, 0, st>>>(w.wv.p, n, w.Vb.p + (int64_t)(j + 1) * n, vst,
                                                                   w.pscal.p, n, rmod, nm));
      if (!more) break;
    }
    // x += Z y for every pair that ran this cycle
    int nvmax = 0;
    for (int64_t q = 0; q < P; ++q) {
      for (int i = 0; i < kMaxBasis; ++i) w.h_py[q * kMaxBasis + i] = make_double2(0, 0);
      w.h_pact[q] = open[q];
      if (!open[q]) continue;
      const int k = ncol[q];
      nvmax = std::max(nvmax, k);
      std::vector<cd> y(k);
      const cd* Hs = H[q].data();
      for (int i = k - 1; i >= 0; --i) {
        cd t = g[q][i];
        for (int c = i + 1; c < k; ++c) t -= Hs[c * (RST + 1) + i] * y[c];
        y[i] = t / Hs[i * (RST + 1) + i];
      }
      for (int i = 0; i < k; ++i) w.h_py[q * kMaxBasis + i] = make_double2(y[i].real(), y[i].imag());
    }
    ELP_CUDA(cudaMemcpyAsync(w.py.p, w.h_py, sizeof(double2) * P * kMaxBasis, cudaMemcpyHostToDevice, st));
    ELP_CUDA(cudaMemcpyAsync(w.pact.p, w.h_pact, sizeof(int) * P, cudaMemcpyHostToDevice, st));
    PROF_LAUNCH(KC_UPDATE, st, k_combo_seg<<<gv, 256, 0, st>>>(w.Zb.p, zst, n, nvmax, w.py.p, w.x.p, n, rmod, nm,
                                                                w.pact.p));
    rc = residual(0, true);  // w.pact: the pairs that ran this cycle
    if (rc) return rc;
  }
  ELP_CUDA(cudaGetLastError());
  float fms = 0.f;
  cudaEventElapsedTime(&fms, w.ev[0], w.ev[1]);
  ms[0] = fms;
  ms[1] = solve_ms;
  ms[2] = 0.f;
  return ELP_OK;
}

// One batch on one workspace lane (0 or 1), on `stream` (its own when null).
static int solve_lane(Model& m, int precision, int lane, const double* omegas, int n_omega, const double2* f_dev,
                      double2* x_dev, elp_solve_info* info, double tol, cudaStream_t stream, int store) {
  int rc = workspace_ensure(m, precision, n_omega, lane, store);
  if (rc) return rc;
  Workspace& w = lane ? *m.ws_b[precision][lane - 1] : *m.ws[precision];
  cudaStream_t st = stream ? stream : w.stream;
  const int64_t n = m.n;
  const int nm = m.n_members;  // a group: one coefficient table (and frequency) per member and slot
  const bool group = nm > 1;
  if (group && f_dev) { set_error("a group solves its members' own right-hand sides"); return ELP_ERR_ARG; }
  int nonzero = 0;  // group members with a nonzero right-hand side
  for (int s = 0; s < n_omega; ++s)
    for (int k = 0; k < nm; ++k) {
      const double om = omegas[(int64_t)s * nm + k];
      Coef& c = w.h_coef[(int64_t)s * nm + k];
      make_coef(m, om, c);
      if (group) {  // F_k(w) to unit norm: the group's residual then bounds each member's
        const double* q = &m.member_f[3 * k];
        const double f2 = q[0] + q[1] / om + q[2] / (om * om);
        // a power of two near 1 / ||F_k(w)||: scaling and unscaling are exact
        c.fscale = f2 > 0.0 ? std::exp2(-std::round(std::log2(std::sqrt(f2)))) : 1.0;
        if (s == 0 && f2 > 0.0) ++nonzero;
      }
    }
  ELP_CUDA(cudaMemcpyAsync(w.coef.p, w.h_coef, sizeof(Coef) * n_omega * nm, cudaMemcpyHostToDevice, st));
  if (group) {
    const dim3 g((unsigned)std::min<int64_t>((n + 255) / 256, 1024), n_omega);
    PROF_LAUNCH(KC_RHS, st, k_group_rhs<<<g, 256, 0, st>>>(
                                combine_args(m), reinterpret_cast<const double2*>(m.dev->rhs.p),
                                m.has_vn ? reinterpret_cast<const double2*>(m.dev->rhs_vn.p) : nullptr, w.coef.p, n,
                                w.f.p));
    // every scaled ||f_k|| lies in [1/sqrt 2, sqrt 2], so ||r|| / ||f|| <= tol / (2 sqrt K)
    // over the group bounds each member's ||r_k|| / ||f_k|| by tol; members that
    // reach tol on their own are frozen on the way (group_mask)
    w.tol_member = tol;
    tol /= 2.0 * std::sqrt((double)std::max(1, nonzero));
  } else {
    for (int s = 0; s < n_omega; ++s) {
      const double2* src = f_dev ? f_dev + (size_t)s * n : reinterpret_cast<const double2*>(m.dev->rhs.p);
      ELP_CUDA(cudaMemcpyAsync(w.f.p + (size_t)s * n, src, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    }
    if (!f_dev && m.has_vn) {  // the model's F(w) = F + G / w
      const dim3 g((unsigned)std::min<int64_t>((n + 255) / 256, 1024), n_omega);
      PROF_LAUNCH(KC_RHS, st, k_add_vn<<<g, 256, 0, st>>>(reinterpret_cast<const double2*>(m.dev->rhs_vn.p), w.coef.p,
                                                          n, w.f.p));
    }
  }
  const double tol_member = group ? w.tol_member : tol;
  // the tensor-core timeout flag reports this batch only
  ELP_CUDA(cudaMemsetAsync(w.tc_err.p, 0, sizeof(int), st));
  int iters = 0;
  float ms[3] = {0, 0, 0};
  if (precision == ELP_MIXED && group) rc = run_gmres_group<float>(m, w, n_omega, w.tol_member, 12, st, ms);
  else if (precision == ELP_MIXED) rc = run_gmres<float>(m, w, n_omega, tol, 12, st, ms);
  else rc = run_batch<double>(m, w, n_omega, tol, 8, st, &iters, ms);
  if (rc) return rc;
  if (group) {  // each member's own true residual (no rows masked), then its solution at its own scale
    for (int s = 0; s < n_omega; ++s) w.h_active[s] = 1;
    ELP_CUDA(cudaMemcpyAsync(w.active.p, w.h_active, sizeof(int) * n_omega, cudaMemcpyHostToDevice, st));
    const CombineArgs Ag = combine_args(m);
    // the mixed path's residual rows are already every pair's true residual (a
    // pair's rows were last computed after its x last changed); the plain
    // path's refinement zeroed the rows of the members it froze
    if (precision != ELP_MIXED)
      PROF_LAUNCH(KC_RESIDUAL, st, k_residual<<<dim3((unsigned)w.nparts, n_omega), 256, 0, st>>>(
                                       Ag, w.coef.p, m.dev->row_ptr.p, m.dev->col_idx.p, n, w.x.p, w.f.p, w.r.p,
                                       w.partial.p, w.nparts, w.active.p, 0));
    PROF_LAUNCH(KC_NORMS, st, k_member_norms<<<dim3(nm, n_omega), 256, 0, st>>>(m.dev->member_off.p, nm, n, w.r.p,
                                                                                  w.f.p, w.mnorms.p));
    const dim3 g((unsigned)std::min<int64_t>((n + 255) / 256, 1024), n_omega);
    PROF_LAUNCH(KC_UPDATE, st, k_group_unscale<<<g, 256, 0, st>>>(combine_args(m), w.coef.p, n, w.x.p));
    ELP_CUDA(cudaMemcpyAsync(w.h_mnorms, w.mnorms.p, sizeof(double) * 2 * n_omega * nm, cudaMemcpyDeviceToHost, st));
    tol = tol_member;
  }
  if (x_dev) ELP_CUDA(cudaMemcpyAsync(x_dev, w.x.p, sizeof(double2) * n * n_omega, cudaMemcpyDeviceToDevice, st));
  ELP_CUDA(cudaMemcpyAsync(w.h_stats, w.stats.p, sizeof(unsigned long long) * 4 * n_omega, cudaMemcpyDeviceToHost, st));
  int tcerr = 0;
  ELP_CUDA(cudaMemcpyAsync(&tcerr, w.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  ELP_CUDA(cudaStreamSynchronize(st));
  prof_resolve();
  if (tcerr) {
    set_error("a tensor-core Schur update gave up waiting for its MMAs");
    return ELP_ERR_CUDA;
  }
  bool ok = true, singular = false;
  for (int sk = 0; sk < n_omega * nm; ++sk) {
    const int s = sk / nm;  // slot; a group reports each member (info[s * nm + k])
    const double* nr = group ? w.h_mnorms + 2 * sk : w.h_norms + 2 * s;
    double fn = nr[1];
    double rel = fn > 0 ? std::sqrt(nr[0] / fn) : std::sqrt(nr[0]);
    if (!(rel <= tol)) {
      ok = false;
      // a zero pivot the static-pivot floor stood in for, and the refinement could not recover
      if (w.h_stats[4 * s + 0] > 0) singular = true;
    }
    if (info) {
      elp_solve_info& I = info[sk];
      I.rel_residual = rel;
      double umax, amax;
      unsigned long long b1 = w.h_stats[4 * s + 1], b3 = w.h_stats[4 * s + 3];
      memcpy(&umax, &b1, 8);
      memcpy(&amax, &b3, 8);
      I.growth = amax > 0 ? umax / amax : 0.0;
      I.iterations = w.iters[s];
      I.static_pivots = (int)w.h_stats[4 * s + 0];
      I.converged = rel <= tol ? 1 : 0;
      I.ms_factor = ms[0] / n_omega;
      I.ms_solve = ms[1] / n_omega;
      I.ms_refine = ms[2] / n_omega;
      I.ms_combine = 0.0;
    }
  }
  if (singular) {
    set_error("zero pivot: the static-pivot floor replaced it and the refinement did not converge "
              "(singular system at this frequency)");
    return ELP_ERR_SINGULAR;
  }
  if (!ok) {
    set_error("iterative refinement did not reach the requested relative residual");
    return ELP_ERR_NOCONV;
  }
  return ELP_OK;
}

int numeric_solve_lane(Model& m, int precision, int lane, const double* omegas, int n_omega, const double2* f_dev,
                       double2* x_dev, elp_solve_info* info, double tol, cudaStream_t stream, int store) {
  if (n_omega <= 0) return ELP_OK;
  if (n_omega > kMaxSlots) { set_error("batch larger than the slot limit"); return ELP_ERR_ARG; }
  if (lane < 0 || lane > 3) { set_error("workspace lane out of range"); return ELP_ERR_ARG; }
  for (int64_t s = 0; s < (int64_t)n_omega * m.n_members; ++s)
    if (!(omegas[s] > 0.0)) { set_error("angular frequency must be > 0"); return ELP_ERR_ARG; }
  return solve_lane(m, precision, lane, omegas, n_omega, f_dev, x_dev, info, tol, stream, store);
}

const double2* lane_solution(const Model& m, int precision, int lane) {
  const std::unique_ptr<Workspace>& W = lane ? m.ws_b[precision][lane - 1] : m.ws[precision];
  return W ? W->x.p : nullptr;
}

int64_t model_array_bytes(const Model& m) {
  const int64_t groups = std::max<int64_t>(1, (int64_t)m.groups.size());
  // row_ptr, col_idx, cls, diag, VK, VM, VKg, rhs (+ vn), bc rows, coordinates, element lists
  int64_t b = m.nnz * (4 + 1 + 8 + 8 + 8 * (groups - 1)) + (m.n + 1) * 4 + m.n * (4 + 16 + (m.has_vn ? 16 : 0));
  b += (int64_t)m.bc_rows.size() * 4 + m.n_nodes * (24 + 3 * 4);
  for (const Block& B : m.blocks) b += (int64_t)B.conn.size() * 4 + B.n_elements * 2;
  b += (int64_t)m.interfaces.size() * (16 * 4 + 8 + 4 * 4);
  if (m.sym) {  // symbolic maps: per-entry arena offsets, front lists, extend-add maps
    const Symbolic& S = *m.sym;
    // per entry: local offset, owner front, row, scatter order
    b += (int64_t)S.entry_local.size() * (8 + 4 + 4 + 4) + (int64_t)S.front_dofs.size() * 4 +
         (int64_t)S.parent_map.size() * 4;
    b += (int64_t)S.fronts.size() * (8 * 4 + 8 * 4 + 4 * 4);
  }
  return b;
}

// Batches of kSplitMin or more frequencies are solved in parts on several
// workspace lanes at once (one host thread and stream per lane): the top of
// the assembly tree is latency-bound (one CTA per front and frequency), so
// one part's top levels overlap another part's throughput-bound lower levels.
// Every frequency slot is computed independently, so the results do not
// depend on the split. Lanes: 4, parts of >= 8 frequencies (ELP_LANES = 1..4;
// 32 frequencies per step: 2 lanes 105.7, 3 lanes 107.3, 4 lanes 108.6
// solves/s); not split while kernel profiling is on.
constexpr int kSplitMin = 16;

int numeric_solve_batch(Model& m, int precision, const double* omegas, int n_omega, const double2* f_dev,
                        double2* x_dev, elp_solve_info* info, double tol, cudaStream_t user_stream,
                        int max_lanes, int store) {
  if (n_omega <= 0) return ELP_OK;
  if (n_omega > kMaxSlots) { set_error("batch larger than the slot limit"); return ELP_ERR_ARG; }
  const int nm = m.n_members;  // a group: omegas and info hold one entry per member and slot
  for (int64_t s = 0; s < (int64_t)n_omega * nm; ++s)
    if (!(omegas[s] > 0.0)) { set_error("angular frequency must be > 0"); return ELP_ERR_ARG; }
  const int lanes = std::min({resolved_tuning(m).lanes, max_lanes, std::max(1, n_omega / (kSplitMin / 2))});
  if (lanes < 2 || n_omega < kSplitMin || prof_on())
    return solve_lane(m, precision, 0, omegas, n_omega, f_dev, x_dev, info, tol, user_stream, store);
  const int64_t n = m.n;
  int first[5];
  for (int l = 0; l <= lanes; ++l) first[l] = (int)((int64_t)n_omega * l / lanes);
  const int part_max = first[1] - first[0] + 1;
  for (int l = 0; l < lanes; ++l) {
    int rc = workspace_ensure(m, precision, part_max, l, store);
    if (rc) return rc;
  }
  // every lane starts after the work already queued on the caller's stream
  cudaEvent_t ev;
  ELP_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  ELP_CUDA(cudaEventRecord(ev, user_stream));
  for (int l = 0; l < lanes; ++l) {
    Workspace& w = l ? *m.ws_b[precision][l - 1] : *m.ws[precision];
    ELP_CUDA(cudaStreamWaitEvent(w.stream, ev, 0));
  }
  int dev = 0;
  cudaGetDevice(&dev);
  int rcs[4] = {ELP_OK, ELP_OK, ELP_OK, ELP_OK};
  std::string errs[4];
  auto run = [&](int l) {
    try {
      cudaSetDevice(dev);
      const int a = first[l], c = first[l + 1] - first[l];
      rcs[l] = solve_lane(m, precision, l, omegas + (size_t)a * nm, c, f_dev ? f_dev + (size_t)a * n : nullptr,
                          x_dev + (size_t)a * n, info ? info + (size_t)a * nm : nullptr, tol, nullptr, store);
    } catch (const std::exception& e) {
      rcs[l] = ELP_ERR_CUDA;
      set_error(std::string("solve lane: ") + e.what());
    }
    if (rcs[l]) errs[l] = get_error();
  };
  std::vector<std::thread> threads;
  for (int l = 1; l < lanes; ++l) threads.emplace_back(run, l);
  run(0);
  for (auto& t : threads) t.join();
  cudaEventDestroy(ev);
  // each lane synchronised its stream before returning: the results are complete
  // solutions and infos of every lane are complete; a frequency that did not
  // reach the tolerance (ELP_ERR_NOCONV, or ELP_ERR_SINGULAR with static
  // pivots) is reported with the results, any other error first
  int soft = ELP_OK;
  for (int l = 0; l < lanes; ++l) {
    if (rcs[l] == ELP_ERR_NOCONV || rcs[l] == ELP_ERR_SINGULAR) {
      if (soft != ELP_ERR_SINGULAR) { soft = rcs[l]; set_error(errs[l]); }
    } else if (rcs[l]) {
      set_error(errs[l]);
      return rcs[l];
    }
  }
  return soft;
}


// One front update of the mixed path on caller-given fronts (elp_front_update_test).
int front_update_test(int kernel, int p, int b, int step, int slots, float* fronts, int parent_m,
                      const int32_t* pmap, float* parents) {
  constexpr int NB = 32;
  if (kernel < 0 || kernel > 4 || p < 1 || b < 0 || slots < 1 || slots > kMaxSlots || !fronts || step < 0) {
    set_error("bad front update test arguments");
    return ELP_ERR_ARG;
  }
  const bool fused = parents != nullptr;
  if (kernel == 3 && !fused) { set_error("the packed Schur update adds into a parent front"); return ELP_ERR_ARG; }
  if (fused) {
    if (kernel < 2 || !pmap || parent_m < b || b < 1) { set_error("bad parent arguments"); return ELP_ERR_ARG; }
    std::vector<char> seen(parent_m, 0);
    for (int i = 0; i < b; ++i) {
      if (pmap[i] < 0 || pmap[i] >= parent_m || seen[pmap[i]]) { set_error("pmap must be injective into the parent"); return ELP_ERR_ARG; }
      seen[pmap[i]] = 1;
    }
  }
  if (kernel < 2 && step * NB >= p) { set_error("step beyond the pivots"); return ELP_ERR_ARG; }
  int rc = tc_kernel_attributes();
  if (rc) return rc;
  const int64_t m = p + b, mP = fused ? parent_m : 0;
  const int64_t per_slot = m * m + mP * mP;  // complex entries: front, then parent
  DevBuf<float2> arena;
  ELP_CUDA(arena.alloc((size_t)slots * per_slot));
  for (int s = 0; s < slots; ++s) {
    ELP_CUDA(cudaMemcpy(arena.p + s * per_slot, fronts + 2 * s * m * m, sizeof(float2) * m * m, cudaMemcpyHostToDevice));
    if (fused)
      ELP_CUDA(cudaMemcpy(arena.p + s * per_slot + m * m, parents + 2 * s * mP * mP, sizeof(float2) * mP * mP,
                          cudaMemcpyHostToDevice));
  }
  const int32_t h_list[1] = {0}, h_fp[2] = {p, (int32_t)mP}, h_fb[2] = {b, 0}, h_par[2] = {fused ? 1 : -1, -1};
  const int32_t h_zero[2] = {0, 0};
  const int64_t h_off[2] = {0, m * m};
  DevBuf<int32_t> list, fp, fb, par, zero, dmap;
  DevBuf<int64_t> foff, pbase;
  DevBuf<int> err;
  ELP_CUDA(list.upload(h_list, 1));
  ELP_CUDA(fp.upload(h_fp, 2));
  ELP_CUDA(fb.upload(h_fb, 2));
  ELP_CUDA(par.upload(h_par, 2));
  ELP_CUDA(zero.upload(h_zero, 2));
  ELP_CUDA(foff.upload(h_off, 2));
  if (fused) ELP_CUDA(dmap.upload(pmap, b));
  ELP_CUDA(err.alloc(1));
  ELP_CUDA(cudaMemset(err.p, 0, sizeof(int)));
  LevelArgs L;
  L.list = list.p;
  L.count = 1;
  L.fp = fp.p;
  L.fb = fb.p;
  L.piv_off = zero.p;
  L.foff = foff.p;
  L.arena_size = per_slot;
  L.n = m;
  L.fparent = par.p;
  L.map_off = zero.p;
  L.pmap = fused ? dmap.p : zero.p;
  L.fuse = fused ? 1 : 0;
  cudaStream_t st = 0;
  if (kernel == 0) {
    dim3 g(1, slots, (unsigned)((m - step * NB + 127) / 128));
    k_gemm_tc<NB, 32, false><<<g, kTcThreads, kTcSmemBytes, st>>>(L, arena.p, step, GM_COL, err.p);
  } else if (kernel == 1) {
    dim3 g(1, slots, (unsigned)std::max<int64_t>(1, (m - step * NB - NB + 127) / 128));
    k_gemm_tc<NB, 32, true><<<g, kTcThreads, kTcSmemBytes, st>>>(L, arena.p, step, GM_ROW, err.p);
  } else if (kernel == 2) {
    dim3 g(1, slots, (unsigned)(((b + 127) / 128) * ((b + 63) / 64)));
    if (b > 0) k_gemm_tc<NB, 64, false><<<g, kTcThreads, kTcSmemBytes, st>>>(L, arena.p, 0, GM_SCHUR, err.p);
  } else if (kernel == 4) {  // the same with 128 x 32 tiles
    dim3 g(1, slots, (unsigned)(((b + 127) / 128) * ((b + 31) / 32)));
    if (b > 0) k_gemm_tc<NB, 32, false><<<g, kTcThreads, kTcSmemBytes, st>>>(L, arena.p, 0, GM_SCHUR, err.p);
  } else {
    const int64_t tiles = (b + kSchurTile - 1) / kSchurTile, nch = (p + kTcKC - 1) / kTcKC;
    const int64_t pack_bytes = tiles * nch * (kSchurABlock + kSchurBBlock);
    const int64_t h_pb[1] = {0};
    ELP_CUDA(pbase.upload(h_pb, 1));
    DevBuf<char> pack;
    ELP_CUDA(pack.alloc((size_t)slots * pack_bytes));
    uint32_t* pk = reinterpret_cast<uint32_t*>(pack.p);
    k_pack_schur<NB><<<dim3(1, slots, (unsigned)std::min<int64_t>(65535, 2 * tiles * nch)), 256, 0, st>>>(L, arena.p, pk, pbase.p,
                                                                                               pack_bytes);
    const int64_t gz = std::min<int64_t>(tiles * tiles, std::max<int64_t>(1, (2 * num_sms() + slots - 1) / slots));
    k_schur_tc<NB><<<dim3(1, slots, (unsigned)gz), kSchurThreads, kSchurSmemBytes, st>>>(L, arena.p, pk, pbase.p,
                                                                                         pack_bytes, err.p, 0);
    ELP_CUDA(cudaGetLastError());
    ELP_CUDA(cudaDeviceSynchronize());
  }
  ELP_CUDA(cudaGetLastError());
  ELP_CUDA(cudaDeviceSynchronize());
  int h_err = 0;
  ELP_CUDA(cudaMemcpy(&h_err, err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (h_err) { set_error("a tensor-core wait ran out"); return ELP_ERR_CUDA; }
  for (int s = 0; s < slots; ++s) {
    ELP_CUDA(cudaMemcpy(fronts + 2 * s * m * m, arena.p + s * per_slot, sizeof(float2) * m * m, cudaMemcpyDeviceToHost));
    if (fused)
      ELP_CUDA(cudaMemcpy(parents + 2 * s * mP * mP, arena.p + s * per_slot + m * m, sizeof(float2) * mP * mP,
                          cudaMemcpyDeviceToHost));
  }
  return ELP_OK;
}

}  // namespace elp
