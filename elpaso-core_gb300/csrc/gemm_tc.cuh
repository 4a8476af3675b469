// Tensor-core (tcgen05, kind::tf32) complex Schur updates of FP32 fronts.
//
// C -= A B on sub-blocks of a column-major complex FP32 front, from four
// real products accumulated in tensor memory,
//   D_re = A_re B_re + (-A_im) B_im      (the minus is the negate-A bit)
//   D_im = A_re B_im + A_im B_re,
// with each real operand split into TF32 hi + lo parts (x = hi + lo, both
// rounded to TF32) and hi*hi + hi*lo + lo*hi accumulated in FP32:
// FP32-level products from three TF32 passes ("3xTF32").
//
// One CTA (256 threads) computes a 128 x NT complex tile: MMA M = 128, N = NT,
// K = 8 per instruction. Operands are converted in registers and stored to
// shared memory in the canonical K-major, no-swizzle layout (8-row x 16-byte
// core matrices; LBO = stride between core matrices along K, SBO = stride
// between 8-row groups); each warp writes whole core matrices, so the stores
// are free of bank conflicts. Two shared-memory stages: while the MMAs of
// chunk c run, the CTA stages chunk c + 1; tcgen05.commit arrives on the
// stage's mbarrier, which is waited on (with an iteration bound) before that
// stage is refilled and before the accumulator is read back with tcgen05.ld.
//
// TRANS = false: MMA rows are rows of C (GM_COL, GM_SCHUR);
// TRANS = true:  MMA rows are columns of C (GM_ROW, whose C has only the 32
//                panel rows), computing C^T -= B^T A^T.
#pragma once
#include <cstdint>

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

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

// waits for the phase with an iteration bound; returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t phase) {
  const uint32_t a = smem_u32(mbar);
  for (uint32_t it = 0; it < (1u << 24); ++it) {
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

__device__ __forceinline__ void ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc

constexpr int kTcKC = 16;  // complex K per stage

// one stage: planes [re_hi, re_lo, im_hi, im_lo] of A (128 x KC) and B (NT x KC)
template <int NT>
struct TcStage {
  uint32_t a[4][128 * kTcKC];
  uint32_t b[4][NT * kTcKC];
};
template <int NT>
struct TcSmem {
  TcStage<NT> st[2];
  uint64_t mbar[2];
  uint32_t tmem_base;
};

// word index of (row, k) in a K-major no-swizzle tile with kTcKC words per row
__device__ __forceinline__ int tc_word(int row, int k) {
  return ((row >> 3) * (kTcKC >> 2) + (k >> 2)) * 32 + (row & 7) * 4 + (k & 3);
}

// C -= A B on one front's sub-block, FP32 complex, tcgen05 3xTF32.
template <int NB, int NT, bool TRANS>
__global__ void __launch_bounds__(256) k_gemm_tc(LevelArgs L, float2* __restrict__ arena, int step, int mode,
                                                 int* __restrict__ err) {
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
  constexpr uint32_t kCols = 2 * NT;  // D_re | D_im, a power of two >= 32
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::smem_u32(&sm.tmem_base)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    tc::mbar_init(&sm.mbar[0], 1);
    tc::mbar_init(&sm.mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = sm.tmem_base;
  constexpr uint32_t id_pos = tc::idesc_tf32(128, NT, false), id_neg = tc::idesc_tf32(128, NT, true);
  constexpr uint32_t LBO = 128, SBO = (kTcKC / 4) * 128;
  uint32_t phase[2] = {0u, 0u};
  bool pending[2] = {false, false};
  bool ok = true;
  // lane -> element of one 8 x 4 core matrix
  const int cr = lane >> 2, ck = lane & 3;
  for (int tile = blockIdx.z; tile < ntiles && ok; tile += gridDim.z) {
    const int i0 = (tile % tiles_r) * 128;
    const int j0 = (tile / tiles_r) * NT;
    int stage = 0, nchunks = (K + kTcKC - 1) / kTcKC;
    for (int c = 0; c < nchunks && ok; ++c, stage ^= 1) {
      const int kc = c * kTcKC;
      if (pending[stage]) {  // the MMAs that read this stage two chunks ago
        ok = tc::mbar_wait(&sm.mbar[stage], phase[stage]);
        phase[stage] ^= 1u;
        pending[stage] = false;
        if (!ok) break;
      }
      TcStage<NT>& S = sm.st[stage];
      // ---- A planes: 128 x KC, core matrices (16 row groups x 4 k groups) over 8 warps
      for (int cm = warp; cm < 16 * (kTcKC / 4); cm += 8) {
        const int i = (cm / (kTcKC / 4)) * 8 + cr, k = (cm % (kTcKC / 4)) * 4 + ck;
        float2 v = make_float2(0.f, 0.f);
        if (i0 + i < MR && kc + k < K)
          v = !TRANS ? F[(int64_t)(kc + k) * m + ra + i0 + i]     // A = L[ra + i, k]
                     : F[(int64_t)(ca + i0 + i) * m + kc + k];   // B^T: U[k, ca + i]
        const int wd = tc_word(i, k);
        uint32_t h, l;
        tc::split_tf32(v.x, h, l);
        S.a[0][wd] = h;
        S.a[1][wd] = l;
        tc::split_tf32(v.y, h, l);
        S.a[2][wd] = h;
        S.a[3][wd] = l;
      }
      // ---- B planes: NT x KC
      for (int cm = warp; cm < (NT / 8) * (kTcKC / 4); cm += 8) {
        const int j = (cm / (kTcKC / 4)) * 8 + cr, k = (cm % (kTcKC / 4)) * 4 + ck;
        float2 v = make_float2(0.f, 0.f);
        if (j0 + j < NC && kc + k < K)
          v = !TRANS ? F[(int64_t)(ca + j0 + j) * m + kc + k]    // U[k, ca + j]
                     : F[(int64_t)(kc + k) * m + ra + j0 + j];  // A^T: L[ra + j, k]
        const int wd = tc_word(j, k);
        uint32_t h, l;
        tc::split_tf32(v.x, h, l);
        S.b[0][wd] = h;
        S.b[1][wd] = l;
        tc::split_tf32(v.y, h, l);
        S.b[2][wd] = h;
        S.b[3][wd] = l;
      }
      tc::fence_async_smem();
      tc::fence_before();
      __syncthreads();
      tc::fence_after();
      if (tid == 0) {
        uint32_t a[4], b[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) { a[q] = tc::smem_u32(S.a[q]); b[q] = tc::smem_u32(S.b[q]); }
        const uint32_t re = tmem, im = tmem + NT;
#pragma unroll
        for (int ks = 0; ks < kTcKC / 8; ++ks) {
          const uint32_t o = ks * 2 * 128;  // two core matrices per K = 8 step
          auto d = [&](uint32_t base) { return tc::smem_desc(base + o, LBO, SBO); };
          const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
          // D_re += A_re B_re - A_im B_im
          tc::mma_tf32(re, d(a[0]), d(b[0]), id_pos, acc0);
          tc::mma_tf32(re, d(a[0]), d(b[1]), id_pos, 1u);
          tc::mma_tf32(re, d(a[1]), d(b[0]), id_pos, 1u);
          tc::mma_tf32(re, d(a[2]), d(b[2]), id_neg, 1u);
          tc::mma_tf32(re, d(a[2]), d(b[3]), id_neg, 1u);
          tc::mma_tf32(re, d(a[3]), d(b[2]), id_neg, 1u);
          // D_im += A_re B_im + A_im B_re
          tc::mma_tf32(im, d(a[0]), d(b[2]), id_pos, acc0);
          tc::mma_tf32(im, d(a[0]), d(b[3]), id_pos, 1u);
          tc::mma_tf32(im, d(a[1]), d(b[2]), id_pos, 1u);
          tc::mma_tf32(im, d(a[2]), d(b[0]), id_pos, 1u);
          tc::mma_tf32(im, d(a[2]), d(b[1]), id_pos, 1u);
          tc::mma_tf32(im, d(a[3]), d(b[0]), id_pos, 1u);
        }
        tc::commit(&sm.mbar[stage]);
      }
      pending[stage] = true;
    }
    // drain both stages before reading the accumulator
    for (int q = 0; q < 2 && ok; ++q)
      if (pending[q]) {
        ok = tc::mbar_wait(&sm.mbar[q], phase[q]);
        phase[q] ^= 1u;
        pending[q] = false;
      }
    tc::fence_after();
    if (!ok) break;
    // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31, column half w / 4
    const int lg = warp & 3, half = warp >> 2;
    if (half * 32 < NT) {
      float re[32], im[32];
      const uint32_t lane_base = (uint32_t)(32 * lg) << 16;
      tc::ld32(tmem + lane_base + half * 32, re);
      tc::ld32(tmem + lane_base + NT + half * 32, im);
      const int i = i0 + 32 * lg + lane;  // MMA row
      if (i < MR) {
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int j = j0 + half * 32 + q;  // MMA column (complex)
          if (j < NC) {
            float2* dst = !TRANS ? F + (int64_t)(ca + j) * m + ra + i : F + (int64_t)(ca + i) * m + ra + j;
            float2 v = *dst;
            v.x -= re[q];
            v.y -= im[q];
            *dst = v;
          }
        }
      }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
  }
  if (!ok && tid == 0) atomicExch(err, 1);
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
  }
}

}  // namespace elp
