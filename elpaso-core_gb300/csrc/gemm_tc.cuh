// Tensor-core (tcgen05, kind::tf32) complex Schur updates of FP32 fronts.
//
// C -= A B on sub-blocks of a column-major complex FP32 front. Every real
// operand x is split into TF32 parts x = hi + lo (both rounded to TF32) and
// hi*hi + hi*lo + lo*hi is accumulated in FP32 ("3xTF32": FP32-level
// products). The complex product is assembled from real MMAs with M = 128:
//   [D_re | D_im] += A_re [B_re | B_im]        (one MMA of N = 2 NT)
//    D_re         += (-A_im) B_im              (negate-A bit, N = NT)
//    D_im         +=   A_im  B_re              (N = NT)
// so a K = 8 step is 9 MMAs (3 products x 3 split terms).
//
// Operand placement (shared-memory bandwidth, not the tensor pipe, bounds a
// 3xTF32 complex update whose operands all come from shared memory):
//  * A (128 rows x KC) lives in TENSOR memory: each thread converts its row's
//    values in registers and writes the four planes [re_hi, re_lo, im_hi,
//    im_lo] with tcgen05.st; the MMAs read A from TMEM;
//  * B (NT x KC, complex) lives in shared memory once, as the two planes hi
//    and lo of the real 2NT x KC matrix [B_re ; B_im], in the canonical
//    K-major no-swizzle layout (8-row x 16-byte core matrices, LBO = stride
//    between core matrices along K, SBO = stride between 8-row groups); the
//    N = NT MMAs address its B_re or B_im half by an SBO offset.
// Warp roles (288 threads): warp 0 issues the MMAs (one elected thread);
// warps 1..8 are converters. Converter warp w owns TMEM lane quarter w % 4
// (the only lanes it may write) and K half (w - 1) / 4 of every A chunk, and
// a fixed set of B elements. The raw complex values go with cp.async (8-byte
// copies, zero-filled outside the block) into the converters' slots of a
// three-chunk ring in shared memory: each converter copies its own values
// (no cross-thread synchronisation: a thread waits only for its own copy
// groups), except the transposed A, which a warp copies together (lanes
// along the contiguous k) and hands over with __syncwarp. Two MMA stages (TMEM columns for A, shared memory for
// B) are handed over with mbarriers, never with block barriers:
//   full[s]  - one arrival per converter warp: stage s holds a converted chunk;
//   empty[s] - tcgen05.commit of the MMAs that read stage s.
// So the converters prepare chunk c + 1 while the tensor pipe runs chunk c,
// whatever back-pressure the MMA issue meets. Every wait is bounded: a
// timeout sets the error flag, and later waits of the CTA are skipped so it
// finishes quickly (with meaningless values) instead of hanging. The CTA
// synchronises only at tile ends: the epilogue (converter warps, tcgen05.ld
// of the accumulator) must finish before the next tile overwrites it.
//
// TRANS = false: MMA rows are rows of C (GM_COL, GM_SCHUR);
// TRANS = true:  MMA rows are columns of C (GM_ROW, whose C has only the 32
//                panel rows), computing C^T -= B^T A^T.
#pragma once
#include <cstdint>
#include <type_traits>

namespace elp {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor (tcgen05): start, LBO, SBO in 16-byte
// units; bits 46-48 = 0b001; base offset 0; no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor: D = F32, A = B = TF32, both K-major, optional
// negation of A (bit 13), N >> 3, M >> 4
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N, bool neg_a = false) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (neg_a ? (1u << 13) : 0u) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  hi = to_tf32(x);
  lo = to_tf32(x - __uint_as_float(hi));
}

// D (TMEM) += A (TMEM, 128 lanes x 8 columns) * B (shared memory descriptor)
__device__ __forceinline__ void mma_tf32_ta(uint32_t tmem_d, uint32_t tmem_a, uint64_t db, uint32_t idesc,
                                            uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(tmem_d),
      "r"(tmem_a), "l"(db), "r"(idesc), "r"(acc));
}

// the warp's 32 TMEM lanes (one per thread), 8 consecutive 32-bit columns
__device__ __forceinline__ void st8(uint32_t taddr, const uint32_t* v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(v[0]),
               "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
               : "memory");
}
__device__ __forceinline__ void wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

// waits for the phase with an iteration bound; returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t phase, uint32_t limit = 1u << 24) {
  const uint32_t a = smem_u32(mbar);
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc

constexpr int kTcKC = 16;            // complex K per chunk
constexpr int kTcRing = 3;           // chunks in flight per converter thread
constexpr int kTcThreads = 288;      // warp 0: MMA issue; warps 1..8: converters
constexpr uint32_t kTcCols = 256;    // TMEM columns per CTA: D (2 NT) + A (2 stages x 4 planes x KC)
constexpr int kTcSmemBytes = 110 * 1024;  // requested dynamic shared memory: caps residency at 2 CTAs
                                          // per SM, so two 256-column TMEM allocations always fit

template <int NT>
struct TcSmem {
  static constexpr int BPT = NT * kTcKC / 256;  // B elements per converter and chunk
  float2 raw[kTcRing][8 + BPT][256];            // [slot][element][converter]: conflict-free
  uint32_t b[2][2][2 * NT * kTcKC];             // [stage][hi, lo] planes of the real 2NT x KC [B_re ; B_im]
  float ep[NT == 32 ? 4 : 1][2][32][17];        // transposed epilogue: re, im of 32 rows x 16 columns per warp
  uint64_t full[2], empty[2];
  uint32_t tmem_base;
};

// word index of (row, k) in a K-major no-swizzle tile with kTcKC words per row
__device__ __forceinline__ int tc_word(int row, int k) {
  return ((row >> 3) * (kTcKC >> 2) + (k >> 2)) * 32 + (row & 7) * 4 + (k & 3);
}

namespace tc {
// 8-byte asynchronous global -> shared copy; zero-fills when !valid
__device__ __forceinline__ void cp8(void* dst, const void* src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 8 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_ring() { asm volatile("cp.async.wait_group %0;" ::"n"(kTcRing - 1) : "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_u32(mbar)) : "memory");
}
}  // namespace tc

// The update C -= D of a front's Schur complement written into its parent
// instead (extend-add fused): cv[q] = C[i, jb + q] - D[i, jb + q] for one row
// i of the border, q < Q; the parent entry of border (i, j) is
// (pmap[i], pmap[j]). Loads of 8 parent entries are issued together.
template <int Q>
__device__ __forceinline__ void add_into_parent(const LevelArgs& L, float2* arena, int f, int s, int i, int jb,
                                                int ncols, const float2* cv) {
  const int P = L.fparent[f];
  const int64_t mP = L.fp[P] + L.fb[P];
  float2* PF = arena + s * L.arena_size + L.foff[P];
  const int32_t* pm = L.pmap + L.map_off[f];
  const int64_t pi = pm[i];
#pragma unroll
  for (int h = 0; h < Q; h += 8) {
    float2 pv[8];
    int64_t po[8];
#pragma unroll
    for (int t = 0; t < 8; ++t)
      if (jb + h + t < ncols) {
        po[t] = (int64_t)pm[jb + h + t] * mP + pi;
        pv[t] = PF[po[t]];
      }
#pragma unroll
    for (int t = 0; t < 8; ++t)
      if (jb + h + t < ncols) PF[po[t]] = make_float2(pv[t].x + cv[h + t].x, pv[t].y + cv[h + t].y);
  }
}

// C -= A B on one front's sub-block, FP32 complex, tcgen05 3xTF32.
template <int NB, int NT, bool TRANS>
__global__ void __launch_bounds__(kTcThreads, 2) k_gemm_tc(LevelArgs L, float2* __restrict__ arena, int step,
                                                           int mode, int* __restrict__ err) {
  static_assert(NT == 32 || NT == 64, "tile width");
  static_assert(2 * NT + 2 * 4 * kTcKC <= (int)kTcCols, "TMEM budget");
  static_assert(sizeof(TcSmem<NT>) <= kTcSmemBytes, "shared memory");
  static_assert(!TRANS || NT == 32, "transposed tiles are 32 wide");
  constexpr int BPT = TcSmem<NT>::BPT;
  constexpr int TPJ = kTcKC / BPT;  // converters per B row
  extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
  TcSmem<NT>& sm = *reinterpret_cast<TcSmem<NT>*>(tc_smem_raw);
  const int f = L.list[blockIdx.x];
  const int s = blockIdx.y;
  const int p = L.fp[f], m = p + L.fb[f];
  const int k0 = step * NB;
  if (mode != GM_SCHUR && k0 >= p) return;
  const int w = min(NB, p - k0);
  int ra, M, ca, N, K;
  if (!gemm_block(mode, p, m, k0, w, ra, M, ca, N, K)) return;
  const int MR = TRANS ? N : M, NC = TRANS ? M : N;  // MMA rows / columns (complex)
  const int tiles_r = (MR + 127) / 128, tiles_c = (NC + NT - 1) / NT;
  const int ntiles = tiles_r * tiles_c;
  if ((int)blockIdx.z >= ntiles) return;  // uniform per CTA, before any TMEM allocation
  float2* F = arena + s * L.arena_size + L.foff[f];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::smem_u32(&sm.tmem_base)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int q = 0; q < 2; ++q) {
      tc::mbar_init(&sm.full[q], 8);  // one arrival per converter warp
      tc::mbar_init(&sm.empty[q], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = sm.tmem_base;
  const uint32_t tD = tmem, tA = tmem + 2 * NT;  // column offsets
  bool ok = true;
  int gc = 0;  // chunks processed by this CTA over all its tiles: stage gc & 1, phase (gc >> 1) & 1
  // converter roles (warps 1..8): A row 32 (warp % 4) + lane, K half (warp - 1) / 4; B row bj, first k bkf
  const int ct = tid - 32;
  const int arow = 32 * (warp & 3) + lane, akh = ((warp - 1) >> 2) * 8;
  const uint32_t a_lane = (uint32_t)(32 * (warp & 3)) << 16;
  // B row bj and first k bkf of each converter: BPT consecutive k per thread; transposed
  // (B^T = L rows, contiguous along j) a warp owns all 32 rows for BPT k, so copies are 256 B runs
  const int bj = !TRANS ? ct / TPJ : ct % NT, bkf = !TRANS ? (ct % TPJ) * BPT : (ct / NT) * BPT;
  for (int tile = blockIdx.z; tile < ntiles; tile += gridDim.z) {
    const int i0 = (tile % tiles_r) * 128;
    const int j0 = (tile / tiles_r) * NT;
    const int nchunks = (K + kTcKC - 1) / kTcKC;
    if (warp == 0) {
      // ------------------------------------------------ MMA issue
      if (lane == 0) {
        constexpr uint32_t id_w = tc::idesc_tf32(128, 2 * NT, false);  // [D_re | D_im]
        constexpr uint32_t id_p = tc::idesc_tf32(128, NT, false), id_n = tc::idesc_tf32(128, NT, true);
        constexpr uint32_t LBO = 128, SBO = (kTcKC / 4) * 128;
        constexpr uint32_t half_off = (NT / 8) * SBO;  // bytes from [B_re] to [B_im] rows
        for (int c = 0; c < nchunks; ++c) {
          const int g = gc + c, stage = g & 1;
          if (ok) ok = tc::mbar_wait(&sm.full[stage], (g >> 1) & 1);
          tc::fence_after();
          const uint32_t bh = tc::smem_u32(sm.b[stage][0]), bl = tc::smem_u32(sm.b[stage][1]);
          const uint32_t a0 = tA + stage * (4 * kTcKC);
#pragma unroll
          for (int ks = 0; ks < kTcKC / 8; ++ks) {
            const uint32_t o = ks * 2 * 128;  // two core matrices per K = 8 step
            const uint32_t a_rh = a0 + 0 * kTcKC + ks * 8, a_rl = a0 + 1 * kTcKC + ks * 8;
            const uint32_t a_ih = a0 + 2 * kTcKC + ks * 8, a_il = a0 + 3 * kTcKC + ks * 8;
            const uint64_t bh_re = tc::smem_desc(bh + o, LBO, SBO), bl_re = tc::smem_desc(bl + o, LBO, SBO);
            const uint64_t bh_im = tc::smem_desc(bh + o + half_off, LBO, SBO);
            const uint64_t bl_im = tc::smem_desc(bl + o + half_off, LBO, SBO);
            const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
            // [D_re | D_im] += A_re [B_re | B_im]
            tc::mma_tf32_ta(tD, a_rh, bh_re, id_w, acc0);
            tc::mma_tf32_ta(tD, a_rh, bl_re, id_w, 1u);
            tc::mma_tf32_ta(tD, a_rl, bh_re, id_w, 1u);
            // D_re -= A_im B_im
            tc::mma_tf32_ta(tD, a_ih, bh_im, id_n, 1u);
            tc::mma_tf32_ta(tD, a_ih, bl_im, id_n, 1u);
            tc::mma_tf32_ta(tD, a_il, bh_im, id_n, 1u);
            // D_im += A_im B_re
            tc::mma_tf32_ta(tD + NT, a_ih, bh_re, id_p, 1u);
            tc::mma_tf32_ta(tD + NT, a_ih, bl_re, id_p, 1u);
            tc::mma_tf32_ta(tD + NT, a_il, bh_re, id_p, 1u);
          }
          tc::commit(&sm.empty[stage]);
        }
      }
      __syncwarp();
    } else {
      // ------------------------------------------------ converters
      // raw copies of this thread's elements of chunk c into ring slot c % kTcRing
      // copy addresses as 32-bit element offsets from the front base (a front has < 2^31
      // entries), advanced per chunk; bounds are checked only where a chunk crosses K
      const int mK = m * kTcKC;
      const int wrow0 = 32 * (warp & 3), wct0 = 32 * (warp - 1), kq = lane & 7;
      const bool arow_ok = i0 + arow < MR, bj_ok = j0 + bj < NC;
      const int a_base = !TRANS ? akh * m + ra + i0 + arow                              // L[ra + i, k]
                                : (ca + i0 + wrow0 + (lane >> 3)) * m + akh + kq;       // U[k, ca + i]
      const int b_base = !TRANS ? (ca + j0 + bj) * m + bkf                              // U[k, ca + j]
                                : bkf * m + ra + j0 + bj;                               // L[ra + j, k]
      auto issue = [&](int c) {
        if (c < nchunks) {
          const int kc = c * kTcKC;
          const bool full = kc + kTcKC <= K;
          float2(*slot)[256] = sm.raw[c % kTcRing];
          if (!TRANS) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {  // lanes along rows of L: coalesced
              const bool v = arow_ok && (full || kc + akh + q < K);
              tc::cp8(&slot[q][ct], F + (v ? a_base + c * mK + q * m : 0), v);
            }
          } else {
            // B^T rows are U columns: a lane's own 8 values are 64 contiguous bytes of one column,
            // so the warp copies its 32 rows x 8 k together, lanes along k (4 rows per copy), into
            // the slots of the lanes that convert them
#pragma unroll
            for (int it = 0; it < 8; ++it) {
              const int rr = (lane >> 3) + 4 * it;
              const bool v = i0 + wrow0 + rr < MR && (full || kc + akh + kq < K);
              tc::cp8(&slot[kq][wct0 + rr], F + (v ? a_base + 4 * it * m + kc : 0), v);
            }
          }
#pragma unroll
          for (int q = 0; q < BPT; ++q) {
            const bool v = bj_ok && (full || kc + bkf + q < K);
            const int off = !TRANS ? b_base + kc + q : b_base + c * mK + q * m;
            tc::cp8(&slot[8 + q][ct], F + (v ? off : 0), v);
          }
        }
        tc::cp_commit();
      };
#pragma unroll
      for (int c = 0; c < kTcRing; ++c) issue(c);
      for (int c = 0; c < nchunks; ++c) {
        const int g = gc + c, stage = g & 1, slot = c % kTcRing;
        tc::cp_wait_ring();  // this thread's copies of chunk c have landed
        if (TRANS) __syncwarp();  // ... and its warp's: some of its A values were copied by other lanes
        float2 av[8], bv[BPT];
#pragma unroll
        for (int q = 0; q < 8; ++q) av[q] = sm.raw[slot][q][ct];
#pragma unroll
        for (int q = 0; q < BPT; ++q) bv[q] = sm.raw[slot][8 + q][ct];
        if (TRANS) __syncwarp();  // every lane has read the slot before any lane refills it
        // stage free: the MMAs of chunk g - 2 have completed (one lane polls, the warp follows)
        if (g >= 2) {
          if (lane == 0 && ok) ok = tc::mbar_wait(&sm.empty[stage], ((g >> 1) + 1) & 1);
          __syncwarp();
        }
        tc::fence_after();
        {  // A planes into TMEM: columns tA + stage*64 + plane*16 + k
          uint32_t h[4][8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            tc::split_tf32(av[q].x, h[0][q], h[1][q]);
            tc::split_tf32(av[q].y, h[2][q], h[3][q]);
          }
          const uint32_t base = tA + stage * (4 * kTcKC) + akh + a_lane;
#pragma unroll
          for (int pl = 0; pl < 4; ++pl) tc::st8(base + pl * kTcKC, h[pl]);
        }
        {  // B planes: rows bj (re) and NT + bj (im), BPT consecutive k
          using VW = typename std::conditional<BPT == 4, uint4, uint2>::type;
          VW hr, lr, hi, li;
          uint32_t* H = &hr.x; uint32_t* Lr = &lr.x; uint32_t* Hi = &hi.x; uint32_t* Li = &li.x;
#pragma unroll
          for (int q = 0; q < BPT; ++q) {
            tc::split_tf32(bv[q].x, H[q], Lr[q]);
            tc::split_tf32(bv[q].y, Hi[q], Li[q]);
          }
          const int wr = tc_word(bj, bkf), wi = tc_word(NT + bj, bkf);
          *reinterpret_cast<VW*>(&sm.b[stage][0][wr]) = hr;
          *reinterpret_cast<VW*>(&sm.b[stage][1][wr]) = lr;
          *reinterpret_cast<VW*>(&sm.b[stage][0][wi]) = hi;
          *reinterpret_cast<VW*>(&sm.b[stage][1][wi]) = li;
        }
        tc::wait_st();
        tc::fence_async_smem();
        tc::fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&sm.full[stage]);
        // refill the slot read above (its values are in registers), off the path to the MMA warp
        issue(c + kTcRing);
      }
      asm volatile("cp.async.wait_all;" ::: "memory");  // only empty groups remain
      // ---- epilogue: the accumulator is complete when the last chunk's commit has arrived
      const int gl = gc + nchunks - 1;
      if (lane == 0 && ok) ok = tc::mbar_wait(&sm.empty[gl & 1], (gl >> 1) & 1);
      __syncwarp();
      tc::fence_after();
      const int lg = warp & 3, half = (warp - 1) >> 2;
      if (half * 32 < NT) {
        const uint32_t lane_base = (uint32_t)(32 * lg) << 16;
        const int i = i0 + 32 * lg + lane;  // MMA row
#pragma unroll
        for (int part = 0; part < 2; ++part) {  // 16 columns at a time: loads first, then stores
          const int jb = j0 + half * 32 + part * 16;
          if (!TRANS) {  // lanes along rows of C: coalesced; 8 columns at a time
#pragma unroll
            for (int e8 = 0; e8 < 16; e8 += 8) {
              const int jb8 = jb + e8;
              float re[8], im[8];
              tc::ld8(tD + lane_base + half * 32 + part * 16 + e8, re);
              tc::ld8(tD + lane_base + NT + half * 32 + part * 16 + e8, im);
              if (ok && i < MR) {
                float2* dst0 = F + (int64_t)(ca + jb8) * m + ra + i;
                float2 cv[8];
#pragma unroll
                for (int q = 0; q < 8; ++q)
                  if (jb8 + q < NC) cv[q] = dst0[(int64_t)q * m];
#pragma unroll
                for (int q = 0; q < 8; ++q) cv[q] = make_float2(cv[q].x - re[q], cv[q].y - im[q]);
                if (mode == GM_SCHUR && L.fuse) {  // the Schur complement goes into the parent
                  add_into_parent<8>(L, arena, f, s, i, jb8, NC, cv);  // border (i, j) of the Schur complement
                } else {
#pragma unroll
                  for (int q = 0; q < 8; ++q)
                    if (jb8 + q < NC) dst0[(int64_t)q * m] = cv[q];
                }
              }
            }
          } else {
            // C^T: the MMA row i is a column of C, contiguous along j; the warp's 32 x 16 block
            // goes through shared memory so that a half-warp writes 16 contiguous entries
            float(*ep)[32][17] = sm.ep[lg];
#pragma unroll
            for (int c2 = 0; c2 < 2; ++c2) {  // re, then im: 16 accumulator values live at a time
              float v[16];
              tc::ld16(tD + lane_base + c2 * NT + half * 32 + part * 16, v);
#pragma unroll
              for (int q = 0; q < 16; ++q) ep[c2][lane][q] = v[q];
            }
            __syncwarp();
            const int jj = lane & 15, r0 = lane >> 4;
#pragma unroll
            for (int t0 = 0; t0 < 16; t0 += 8) {  // 8 rows per half-warp at a time: loads, then stores
              float2 cv[8];
#pragma unroll
              for (int t = 0; t < 8; ++t) {
                const int ii = i0 + 32 * lg + 2 * (t0 + t) + r0;
                if (ok && ii < MR && jb + jj < NC) cv[t] = F[(int64_t)(ca + ii) * m + ra + jb + jj];
              }
#pragma unroll
              for (int t = 0; t < 8; ++t) {
                const int r = 2 * (t0 + t) + r0, ii = i0 + 32 * lg + r;
                if (ok && ii < MR && jb + jj < NC)
                  F[(int64_t)(ca + ii) * m + ra + jb + jj] =
                      make_float2(cv[t].x - ep[0][r][jj], cv[t].y - ep[1][r][jj]);
              }
            }
            __syncwarp();  // the staging block is rewritten by the next part
          }
        }
      }
    }
    gc += nchunks;
    // the accumulator is read before the next tile's first MMA overwrites it
    tc::fence_before();
    ok = __syncthreads_and(ok);
    tc::fence_after();
  }
  // every commit has been waited on by the epilogue (or a wait timed out, in which
  // case the MMAs that may still run are waited for, bounded, before the release)
  if (!ok && tid == 0) {
    atomicExch(err, 1);
    for (int q = 0; q < 2; ++q) {  // the last chunk committed on stage q
      const int gq = ((gc - 1) & 1) == q ? gc - 1 : gc - 2;
      if (gq >= 0) tc::mbar_wait(&sm.empty[q], (gq >> 1) & 1);
    }
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
  }
}

// ===================================================================== Schur update from packed operands
//
// The Schur complement update GM_SCHUR (C = F[p:m, p:m] -= L21 U12, depth p)
// reads operands that are final once the level's panels are done, so they are
// split into TF32 planes ONCE per level (k_pack_schur) in the exact
// shared-memory layout the MMAs read (K-major, no swizzle, 16-deep chunks):
//   A block (tile row tr, chunk c): L21 rows 128 tr.., 4 planes re_hi, re_lo,
//     im_hi, im_lo of 128 x 16 words (32 KB);
//   B block (tile col tc, chunk c): U12 columns 128 tc.., the 2 planes hi, lo
//     of W = [B_re ; B_im], 256 x 16 words each (32 KB).
// k_schur_tc then needs no converter threads: one thread issues two 1D bulk
// copies (cp.async.bulk, completing on an mbarrier with a byte count) per
// chunk into a three-stage ring, one thread issues the MMAs, all eight warps
// run the epilogue. A 128 x 128 complex tile, per K = 8 step (3xTF32:
// hi*hi + hi*lo + lo*hi), accumulated in 256 TMEM columns:
//   [D_re | D_im] += A_re W          (N = 256)
//    D_re         -= A_im B_im        (N = 128, negate-A, B_im = rows 128.. of W)
//    D_im         += A_im B_re        (N = 128)
// 9 MMAs with the work of 6 of N = 256, and half the B bytes of a layout that
// also stores [-B_im ; B_re].
constexpr int kSchurTile = 128;                  // complex rows and columns of a tile
constexpr int64_t kSchurABlock = 4 * 128 * kTcKC * 4;
constexpr int64_t kSchurBBlock = 2 * 256 * kTcKC * 4;
constexpr uint32_t kSchurCols = 256;
constexpr int kSchurStages = 3;

struct SchurStage {
  uint32_t a[4][128 * kTcKC];
  uint32_t b[2][256 * kTcKC];
};
struct SchurSmem {
  SchurStage st[kSchurStages];
  uint64_t full[kSchurStages], empty[kSchurStages];
  uint64_t acc_full[2], acc_empty[2];
  uint32_t tmem_base;
};
constexpr int kSchurSmemBytes = (int)((sizeof(SchurSmem) + 1023) / 1024 * 1024);

namespace tc {
__device__ __forceinline__ void mma_tf32_ss(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* mbar, uint32_t bytes) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(
                   smem_u32(mbar)), "r"(bytes)
               : "memory");
}
// 1D bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(mbar))
      : "memory");
}
}  // namespace tc

// Packs L21 and U12 of every front of a level and every frequency slot.
// Grid: (fronts, slots, blocks); a CTA of 256 threads writes one block. A
// thread takes one row and 4 consecutive k (one 16-byte row of a core matrix
// per plane): 4 loads, then one 16-byte store per plane, so a warp writes
// whole 128-byte lines.
template <int NB>
__global__ void __launch_bounds__(256) k_pack_schur(LevelArgs L, const float2* __restrict__ arena,
                                                    uint32_t* __restrict__ pack, const int64_t* __restrict__ pack_base,
                                                    int64_t slot_bytes) {
  const int f = L.list[blockIdx.x];
  const int s = blockIdx.y;
  const int p = L.fp[f], b = L.fb[f], m = p + b;
  if (p == 0 || b == 0) return;
  const int tiles = (b + kSchurTile - 1) / kSchurTile, nch = (p + kTcKC - 1) / kTcKC;
  const int nA = tiles * nch;
  const float2* F = arena + s * L.arena_size + L.foff[f];
  char* base = reinterpret_cast<char*>(pack) + s * slot_bytes + pack_base[f];
  // word of (row, k) within a plane, k = 4 kq + (0..3) stored contiguously
  auto row16 = [](int row, int kq) { return ((row >> 3) * (kTcKC >> 2) + kq) * 32 + (row & 7) * 4; };
  // blocks z, z + gridDim.z, ...: the largest fronts have more than 65,535
  for (int blk0 = blockIdx.z; blk0 < 2 * nA; blk0 += gridDim.z) {
  int blk = blk0;
  if (blk < nA) {
    const int tr = blk / nch, c = blk % nch;
    uint32_t* P = reinterpret_cast<uint32_t*>(base + (int64_t)blk * kSchurABlock);
    constexpr int PL = 128 * kTcKC;  // words per plane
    for (int t = threadIdx.x; t < 128 * (kTcKC / 4); t += blockDim.x) {
      const int ii = t % 128, kq = t / 128;  // lanes along the rows of L21: coalesced loads
      const int i = tr * 128 + ii, k0 = c * kTcKC + 4 * kq;
      float2 v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = (i < b && k0 + q < p) ? F[(int64_t)(k0 + q) * m + p + i] : make_float2(0.f, 0.f);
      uint4 rh, rl, ih, il;
      tc::split_tf32(v[0].x, rh.x, rl.x); tc::split_tf32(v[1].x, rh.y, rl.y);
      tc::split_tf32(v[2].x, rh.z, rl.z); tc::split_tf32(v[3].x, rh.w, rl.w);
      tc::split_tf32(v[0].y, ih.x, il.x); tc::split_tf32(v[1].y, ih.y, il.y);
      tc::split_tf32(v[2].y, ih.z, il.z); tc::split_tf32(v[3].y, ih.w, il.w);
      const int wd = row16(ii, kq);
      *reinterpret_cast<uint4*>(&P[0 * PL + wd]) = rh;
      *reinterpret_cast<uint4*>(&P[1 * PL + wd]) = rl;
      *reinterpret_cast<uint4*>(&P[2 * PL + wd]) = ih;
      *reinterpret_cast<uint4*>(&P[3 * PL + wd]) = il;
    }
  } else {
    blk -= nA;
    const int tcol = blk / nch, c = blk % nch;
    uint32_t* P = reinterpret_cast<uint32_t*>(base + (int64_t)nA * kSchurABlock + (int64_t)blk * kSchurBBlock);
    constexpr int PL = 256 * kTcKC;  // words per plane
    for (int t = threadIdx.x; t < 128 * (kTcKC / 4); t += blockDim.x) {
      const int kq = t % (kTcKC / 4), jj = t / (kTcKC / 4);  // 4 lanes cover 16 k of a U12 column: coalesced
      const int j = tcol * 128 + jj, k0 = c * kTcKC + 4 * kq;
      float2 v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = (j < b && k0 + q < p) ? F[(int64_t)(p + j) * m + k0 + q] : make_float2(0.f, 0.f);
      uint4 rh, rl, ih, il;
      tc::split_tf32(v[0].x, rh.x, rl.x); tc::split_tf32(v[1].x, rh.y, rl.y);
      tc::split_tf32(v[2].x, rh.z, rl.z); tc::split_tf32(v[3].x, rh.w, rl.w);
      tc::split_tf32(v[0].y, ih.x, il.x); tc::split_tf32(v[1].y, ih.y, il.y);
      tc::split_tf32(v[2].y, ih.z, il.z); tc::split_tf32(v[3].y, ih.w, il.w);
      const int w_re = row16(jj, kq), w_im = row16(128 + jj, kq);  // W = [B_re ; B_im]
      *reinterpret_cast<uint4*>(&P[0 * PL + w_re]) = rh;
      *reinterpret_cast<uint4*>(&P[1 * PL + w_re]) = rl;
      *reinterpret_cast<uint4*>(&P[0 * PL + w_im]) = ih;
      *reinterpret_cast<uint4*>(&P[1 * PL + w_im]) = il;
    }
  }
  }
}

// C -= L21 U12 over the 128 x 128 complex tiles of one front and frequency:
// CTA blockIdx.z takes tiles z, z + gridDim.z, ... (one CTA per SM: 197 KB of
// shared memory). Warp 0 lane 0 copies the operand chunks into the
// three-stage ring, warp 1 lane 0 issues the MMAs, warps 2..9 run the
// epilogue (warp w reads TMEM lane quarter w % 4, column half (w - 2) / 4).
// Two accumulators (TMEM columns 0..255 and 256..511) let the epilogue of one
// tile run while the MMAs of the next fill the other:
//   full[st] / empty[st]  - operand stage loaded (bytes) / read by the MMAs (commit);
//   acc_full[a]           - the MMAs of a tile are complete (commit);
//   acc_empty[a]          - the 8 epilogue warps have read accumulator a.
// Every wait is bounded; after a timeout a role stops, the CTA sets the error
// flag and waits (bounded) for its copies and MMAs in flight before the TMEM
// is released. fault != 0 (a host-side test switch, elp_fault_inject) makes
// the producer issue nothing and bounds every wait at 2^14 polls: the MMA
// and epilogue waits then run out with no copy or MMA in flight.
constexpr int kSchurThreads = 320;

// Tile t of a front's tiles x tiles Schur complement, in groups of G tile rows
// walked column by column: the tiles that run at the same time (consecutive t)
// span G row blocks of L21 and about (concurrent / G) column blocks of U12,
// instead of every row block of one column, so fewer operand blocks are read
// from DRAM more than once. The last group may have fewer rows.
__device__ __forceinline__ void schur_tile_rc(int t, int tiles, int G, int& tr, int& tcol) {
  const int grp = t / (G * tiles), idx = t - grp * G * tiles;
  const int r0 = grp * G, rows = min(G, tiles - r0);
  tcol = idx / rows;
  tr = r0 + idx % rows;
}

template <int NB>
__global__ void __launch_bounds__(kSchurThreads, 1) k_schur_tc(LevelArgs L, float2* __restrict__ arena,
                                                               const uint32_t* __restrict__ pack,
                                                               const int64_t* __restrict__ pack_base,
                                                               int64_t slot_bytes, int* __restrict__ err,
                                                               int fault) {
  extern __shared__ __align__(1024) unsigned char schur_smem_raw[];
  SchurSmem& sm = *reinterpret_cast<SchurSmem*>(schur_smem_raw);
  const int f = L.list[blockIdx.x];
  const int s = blockIdx.y;
  const int p = L.fp[f], b = L.fb[f], m = p + b;
  if (p == 0 || b == 0) return;
  const int tiles = (b + kSchurTile - 1) / kSchurTile, nch = (p + kTcKC - 1) / kTcKC;
  const int ntile = tiles * tiles;
  if ((int)blockIdx.z >= ntile) return;  // uniform per CTA, before any TMEM allocation
  const int nmine = (ntile - 1 - (int)blockIdx.z) / (int)gridDim.z + 1;
  // about half the CTAs of a front and slot run at once (two waves per launch):
  // groups of ~sqrt of that many tile rows
  const int G = max(1, min(tiles, (int)(sqrtf(0.5f * (float)gridDim.z) + 0.5f)));
  const char* base = reinterpret_cast<const char*>(pack) + s * slot_bytes + pack_base[f];
  const char* Abase = base;
  const char* Bbase = base + (int64_t)tiles * nch * kSchurABlock;
  float2* F = arena + s * L.arena_size + L.foff[f];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::smem_u32(&sm.tmem_base)),
                 "r"(2 * kSchurCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int q = 0; q < kSchurStages; ++q) {
      tc::mbar_init(&sm.full[q], 1);
      tc::mbar_init(&sm.empty[q], 1);
    }
    for (int q = 0; q < 2; ++q) {
      tc::mbar_init(&sm.acc_full[q], 1);
      tc::mbar_init(&sm.acc_empty[q], 8);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = sm.tmem_base;
  bool ok = true;
  const uint32_t lim = fault ? (1u << 14) : (1u << 24);  // poll bound of every wait
  // chunk g (counted over all this CTA's tiles) uses stage g % kSchurStages, and
  // its use g / kSchurStages of the stage completes mbarrier phase (g / kSchurStages) & 1;
  // tile j uses accumulator j & 1, whose use j / 2 completes phase (j / 2) & 1
  int issued = 0, mma_chunks = 0, mma_tiles = 0;
  if (warp == 0 && lane == 0) {
    // ------------------------------------------------ producer
    int g = 0;
    for (int j = 0; j < nmine && ok && !fault; ++j) {
      const int t = (int)blockIdx.z + j * (int)gridDim.z;
      int tr, tcol;
      schur_tile_rc(t, tiles, G, tr, tcol);
      const char* Ab = Abase + (int64_t)(tr * nch) * kSchurABlock;
      const char* Bb = Bbase + (int64_t)(tcol * nch) * kSchurBBlock;
      for (int c = 0; c < nch; ++c, ++g) {
        const int st = g % kSchurStages;
        if (g >= kSchurStages && ok) ok = tc::mbar_wait(&sm.empty[st], ((g / kSchurStages) + 1) & 1, lim);
        if (!ok) break;
        tc::mbar_expect_tx(&sm.full[st], (uint32_t)(kSchurABlock + kSchurBBlock));
        tc::bulk_g2s(&sm.st[st].a[0][0], Ab + (int64_t)c * kSchurABlock, (uint32_t)kSchurABlock, &sm.full[st]);
        tc::bulk_g2s(&sm.st[st].b[0][0], Bb + (int64_t)c * kSchurBBlock, (uint32_t)kSchurBBlock, &sm.full[st]);
        issued = g + 1;
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ------------------------------------------------ MMA issue
    constexpr uint32_t id_w = tc::idesc_tf32(128, 256, false);
    constexpr uint32_t id_p = tc::idesc_tf32(128, 128, false), id_n = tc::idesc_tf32(128, 128, true);
    constexpr uint32_t LBO = 128, SBO = (kTcKC / 4) * 128;
    constexpr uint32_t half_off = (128 / 8) * SBO;  // bytes from the B_re rows of W to its B_im rows
    int g = 0;
    for (int j = 0; j < nmine && ok; ++j) {
      const int acc = j & 1;
      const uint32_t D = tmem + (uint32_t)acc * kSchurCols;
      if (j >= 2) ok = tc::mbar_wait(&sm.acc_empty[acc], ((j / 2) + 1) & 1, lim);  // epilogue of tile j - 2 read it
      tc::fence_after();
      for (int c = 0; c < nch && ok; ++c, ++g) {
        const int st = g % kSchurStages;
        ok = tc::mbar_wait(&sm.full[st], (g / kSchurStages) & 1, lim);
        if (!ok) break;
        tc::fence_after();
        uint32_t a[4], w[2];
#pragma unroll
        for (int q = 0; q < 4; ++q) a[q] = tc::smem_u32(sm.st[st].a[q]);
#pragma unroll
        for (int q = 0; q < 2; ++q) w[q] = tc::smem_u32(sm.st[st].b[q]);
#pragma unroll
        for (int ks = 0; ks < kTcKC / 8; ++ks) {
          const uint32_t o = ks * 2 * 128;  // two core matrices per K = 8 step
          auto d = [&](uint32_t x) { return tc::smem_desc(x + o, LBO, SBO); };
          const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
          // [D_re | D_im] += A_re [B_re | B_im]
          tc::mma_tf32_ss(D, d(a[0]), d(w[0]), id_w, acc0);  // A_re_hi W_hi
          tc::mma_tf32_ss(D, d(a[0]), d(w[1]), id_w, 1u);    // A_re_hi W_lo
          tc::mma_tf32_ss(D, d(a[1]), d(w[0]), id_w, 1u);    // A_re_lo W_hi
          // D_re -= A_im B_im
          tc::mma_tf32_ss(D, d(a[2]), d(w[0] + half_off), id_n, 1u);
          tc::mma_tf32_ss(D, d(a[2]), d(w[1] + half_off), id_n, 1u);
          tc::mma_tf32_ss(D, d(a[3]), d(w[0] + half_off), id_n, 1u);
          // D_im += A_im B_re
          tc::mma_tf32_ss(D + 128, d(a[2]), d(w[0]), id_p, 1u);
          tc::mma_tf32_ss(D + 128, d(a[2]), d(w[1]), id_p, 1u);
          tc::mma_tf32_ss(D + 128, d(a[3]), d(w[0]), id_p, 1u);
        }
        tc::commit(&sm.empty[st]);
        mma_chunks = g + 1;
      }
      if (!ok) break;
      tc::commit(&sm.acc_full[acc]);
      mma_tiles = j + 1;
    }
  } else if (warp >= 2) {
    // ------------------------------------------------ epilogue
    const int lg = warp & 3, half = (warp - 2) >> 2;  // TMEM lane quarter, 64-column half of the tile
    const uint32_t lane_base = (uint32_t)(32 * lg) << 16;
    for (int j = 0; j < nmine; ++j) {
      const int acc = j & 1;
      const int t = (int)blockIdx.z + j * (int)gridDim.z;
      int tr, tcol;
      schur_tile_rc(t, tiles, G, tr, tcol);
      if (lane == 0 && ok) ok = tc::mbar_wait(&sm.acc_full[acc], (j / 2) & 1, lim);
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      tc::fence_after();
      const uint32_t D = tmem + lane_base + (uint32_t)acc * kSchurCols;
      const int i = tr * kSchurTile + 32 * lg + lane;  // row of C (within the border block)
#pragma unroll
      for (int part = 0; part < 4; ++part) {  // 16 complex columns at a time: loads first, then stores
        const int jb = tcol * kSchurTile + half * 64 + part * 16;
        float re[16], im[16];
        tc::ld16(D + half * 64 + part * 16, re);
        tc::ld16(D + 128 + half * 64 + part * 16, im);
        if (i < b) {
          float2* dst0 = F + (int64_t)(p + jb) * m + p + i;
          float2 cv[16];
#pragma unroll
          for (int q = 0; q < 16; ++q)
            if (jb + q < b) cv[q] = dst0[(int64_t)q * m];
#pragma unroll
          for (int q = 0; q < 16; ++q) cv[q] = make_float2(cv[q].x - re[q], cv[q].y - im[q]);
          if (L.fuse) {
            add_into_parent<16>(L, arena, f, s, i, jb, b, cv);
          } else {
#pragma unroll
            for (int q = 0; q < 16; ++q)
              if (jb + q < b) dst0[(int64_t)q * m] = cv[q];
          }
        }
      }
      // this warp has read accumulator acc (ld16 waits for its loads)
      tc::fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&sm.acc_empty[acc]);
    }
  }
  const bool any_fail = __syncthreads_or(!ok);
  if (any_fail) {
    // a wait ran out: copies and MMAs of the last chunks may still be in flight;
    // wait (bounded) for their barriers before the shared memory and TMEM go away
    if (tid == 0) {
      atomicExch(err, 1);
      for (int g = (issued > kSchurStages ? issued - kSchurStages : 0); g < issued; ++g)
        tc::mbar_wait(&sm.full[g % kSchurStages], (g / kSchurStages) & 1, lim);
    } else if (tid == 32) {
      for (int g = (mma_chunks > kSchurStages ? mma_chunks - kSchurStages : 0); g < mma_chunks; ++g)
        tc::mbar_wait(&sm.empty[g % kSchurStages], (g / kSchurStages) & 1, lim);
      for (int j = (mma_tiles > 2 ? mma_tiles - 2 : 0); j < mma_tiles; ++j)
        tc::mbar_wait(&sm.acc_full[j & 1], (j / 2) & 1, lim);
    }
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kSchurCols) : "memory");
  }
}

}  // namespace elp
