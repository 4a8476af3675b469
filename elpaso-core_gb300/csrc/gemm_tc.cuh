// Tensor-core (tcgen05, kind::tf32) complex Schur updates of FP32 fronts.
//
// C -= A B on sub-blocks of a column-major complex FP32 front, with the
// complex product written as one real GEMM on real blocks:
//   [C_re | C_im] = [A_re  A_im] . [[ B_re, B_im],
//                                   [-B_im, B_re]]
// and each real operand split into TF32 hi + lo parts (x = hi + lo, both
// rounded to TF32), accumulating hi*hi + hi*lo + lo*hi in FP32 in tensor
// memory: FP32-level products from three TF32 passes ("3xTF32").
//
// One CTA (256 threads) computes a 128 x NT complex tile: MMA M = 128 rows,
// N = 2 NT real columns, K = 8 per instruction. Operands are converted in
// registers and stored to shared memory in the canonical K-major,
// no-swizzle layout (8-row x 16-byte core matrices; LBO = stride between
// core matrices along K, SBO = stride between 8-row groups); thread 0 issues
// the MMAs; tcgen05.commit arrives on an mbarrier that every thread waits on
// (with an iteration bound) before the shared buffers are refilled or the
// accumulator is read back with tcgen05.ld.
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

// instruction descriptor: D = F32, A = B = TF32, both K-major, N >> 3, M >> 4
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
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

// byte offset of (row, k) in a K-major no-swizzle tile with KT 32-bit elements per row
__device__ __forceinline__ uint32_t kmajor_off(int row, int k, int KT) {
  return (uint32_t)(((row >> 3) * (KT >> 2) + (k >> 2)) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

}  // namespace tc

constexpr int kTcKC = 16;               // complex K per chunk
constexpr int kTcKT = 2 * kTcKC;        // real K per chunk (real and imaginary blocks)

template <int NT>
struct TcSmem {
  uint32_t a_hi[128 * kTcKT], a_lo[128 * kTcKT];            // 128 rows x KT
  uint32_t b_hi[2 * NT * kTcKT], b_lo[2 * NT * kTcKT];      // 2 NT rows x KT
  uint64_t mbar;
  uint32_t tmem_base;
};

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
  // MMA-row extent MR and MMA-column extent NC (complex)
  const int MR = TRANS ? N : M, NC = TRANS ? M : N;
  const int tiles_r = (MR + 127) / 128, tiles_c = (NC + NT - 1) / NT;
  const int ntiles = tiles_r * tiles_c;
  if ((int)blockIdx.z >= ntiles) return;  // uniform per CTA
  float2* F = arena + s * L.arena_size + L.foff[f];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr uint32_t kCols = 2 * NT < 32 ? 32 : 2 * NT;   // TMEM columns (power of two >= 32)
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::smem_u32(&sm.tmem_base)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    tc::mbar_init(&sm.mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = sm.tmem_base;
  constexpr uint32_t idesc = tc::idesc_tf32(128, 2 * NT);
  uint32_t phase = 0;
  bool ok = true;
  for (int tile = blockIdx.z; tile < ntiles && ok; tile += gridDim.z) {
    const int i0 = (tile % tiles_r) * 128;   // MMA row origin
    const int j0 = (tile / tiles_r) * NT;    // MMA column origin (complex)
    for (int kc = 0; kc < K; kc += kTcKC) {
      // ---- stage P (128 x KC complex) as [re | im] real blocks, hi/lo
      for (int t = tid; t < 128 * kTcKC; t += 256) {
        int i, k;
        if (!TRANS) { i = t % 128; k = t / 128; }   // column-major source: i contiguous
        else { k = t % kTcKC; i = t / kTcKC; }       // U row segments: k contiguous
        float2 v = make_float2(0.f, 0.f);
        if (i0 + i < MR && kc + k < K) {
          v = !TRANS ? F[(int64_t)(kc + k) * m + ra + i0 + i]        // A = L[ra + i, k]
                     : F[(int64_t)(ca + i0 + i) * m + kc + k];      // B^T: U[k, ca + i]
        }
        uint32_t h, l;
        tc::split_tf32(v.x, h, l);
        sm.a_hi[tc::kmajor_off(i, k, kTcKT) >> 2] = h;
        sm.a_lo[tc::kmajor_off(i, k, kTcKT) >> 2] = l;
        tc::split_tf32(v.y, h, l);
        sm.a_hi[tc::kmajor_off(i, kTcKC + k, kTcKT) >> 2] = h;
        sm.a_lo[tc::kmajor_off(i, kTcKC + k, kTcKT) >> 2] = l;
      }
      // ---- stage Q (NT x KC complex) as [[re, -im], [im, re]] real blocks
      for (int t = tid; t < NT * kTcKC; t += 256) {
        int j, k;
        if (!TRANS) { k = t % kTcKC; j = t / kTcKC; }  // U[k, ca + j]: k contiguous
        else { j = t % NT; k = t / NT; }                 // A^T: L[ra + j, k]: j contiguous
        float2 v = make_float2(0.f, 0.f);
        if (j0 + j < NC && kc + k < K) {
          v = !TRANS ? F[(int64_t)(ca + j0 + j) * m + kc + k]
                     : F[(int64_t)(kc + k) * m + ra + j0 + j];
        }
        uint32_t rh, rl, ih, il, nh, nl;
        tc::split_tf32(v.x, rh, rl);
        tc::split_tf32(v.y, ih, il);
        tc::split_tf32(-v.y, nh, nl);
        sm.b_hi[tc::kmajor_off(j, k, kTcKT) >> 2] = rh;
        sm.b_lo[tc::kmajor_off(j, k, kTcKT) >> 2] = rl;
        sm.b_hi[tc::kmajor_off(j, kTcKC + k, kTcKT) >> 2] = nh;
        sm.b_lo[tc::kmajor_off(j, kTcKC + k, kTcKT) >> 2] = nl;
        sm.b_hi[tc::kmajor_off(NT + j, k, kTcKT) >> 2] = ih;
        sm.b_lo[tc::kmajor_off(NT + j, k, kTcKT) >> 2] = il;
        sm.b_hi[tc::kmajor_off(NT + j, kTcKC + k, kTcKT) >> 2] = rh;
        sm.b_lo[tc::kmajor_off(NT + j, kTcKC + k, kTcKT) >> 2] = rl;
      }
      tc::fence_async_smem();
      tc::fence_before();
      __syncthreads();
      tc::fence_after();
      if (tid == 0) {
        const uint32_t lbo = 128, sbo = (kTcKT / 4) * 128;
        const uint32_t ah = tc::smem_u32(sm.a_hi), al = tc::smem_u32(sm.a_lo);
        const uint32_t bh = tc::smem_u32(sm.b_hi), bl = tc::smem_u32(sm.b_lo);
#pragma unroll
        for (int ks = 0; ks < kTcKT / 8; ++ks) {
          const uint32_t ko = ks * 2 * 128;  // two core matrices per K = 8 step
          const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
          tc::mma_tf32(tmem, tc::smem_desc(ah + ko, lbo, sbo), tc::smem_desc(bh + ko, lbo, sbo), idesc, acc);
          tc::mma_tf32(tmem, tc::smem_desc(ah + ko, lbo, sbo), tc::smem_desc(bl + ko, lbo, sbo), idesc, 1u);
          tc::mma_tf32(tmem, tc::smem_desc(al + ko, lbo, sbo), tc::smem_desc(bh + ko, lbo, sbo), idesc, 1u);
        }
        tc::commit(&sm.mbar);
      }
      ok = tc::mbar_wait(&sm.mbar, phase);
      phase ^= 1u;
      tc::fence_after();
      if (!ok) break;
    }
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
