// Allocation-free residual check: r = f - A(w) x and ||r||_2 / ||f||_2 for
// up to ELP_NOALLOC_MAX_OMEGA frequencies, without any device allocation.
//
// Some callers cannot call cudaMalloc while they run: a process whose device
// memory is owned by another framework's pool or a fixed budget that it
// cannot grow, an embedding (a plugin inside a larger solver, a real-time
// host) that forbids allocation after start-up, or a loop that must not pay
// the implicit device-wide synchronisation a cudaMalloc/cudaFree can cause. They still need the FP64 residual check that
// the solve path performs (numeric.cu k_residual / k_norms), whose reduction
// partials and coefficient table normally live in a workspace allocated by
// the library. This variant keeps that scratch in one file-scope device
// array of fixed size instead:
//  - every GPU that loads the library holds kScratchBytes of it until the
//    process exits;
//  - all calls share it and it keeps the last call's contents; what must
//    start at zero is cleared by each call, and calls that overlap on the
//    GPU (different streams or threads at the same time) race on it;
//  - the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (a host-side name is not a device address); make
//    that first call before any stream capture;
//  - it needs an assembled model only (the symbolic phase is not used);
//  - its launches are not counted or timed by elp_profile.
// A call with profiling on still allocates nothing.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "device.cuh"
#include "numeric.cuh"

namespace elp {
namespace {

constexpr int kNoAllocParts = 512;  // reduction blocks per frequency

struct NoAllocScratch {
  Coef coef[ELP_NOALLOC_MAX_OMEGA];
  double partial[ELP_NOALLOC_MAX_OMEGA][kNoAllocParts][2];
  double rel[ELP_NOALLOC_MAX_OMEGA];
};
constexpr size_t kScratchBytes = (sizeof(NoAllocScratch) + 255) / 256 * 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_ptr[64] = {nullptr};

// device address of the scratch array on the current device (set-up once per device)
int scratch_address(NoAllocScratch** out) {
  int dev = 0;
  ELP_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { set_error("device index out of range"); return ELP_ERR_ARG; }
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error(std::string("cudaGetSymbolAddress for the scratch array failed: ") + cudaGetErrorString(e));
      return ELP_ERR_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = static_cast<NoAllocScratch*>(g_scratch_ptr[dev]);
  return ELP_OK;
}

// r = f - A x per row (kRowLanes lanes per row, as the solve path's
// k_residual) and per-block |r|^2, |f|^2 into the scratch
__global__ void k_noalloc_residual(CombineArgs A, NoAllocScratch* sc, const int32_t* __restrict__ row_ptr,
                                   const int32_t* __restrict__ col_idx, int64_t n, const double2* __restrict__ x,
                                   const double2* __restrict__ f, double2* __restrict__ r) {
  const int s = blockIdx.y;
  const Coef c = sc->coef[s];
  const int lane = threadIdx.x & 31, sub = lane & (kRowLanes - 1);
  const double2* xs = x + s * n;
  double rr = 0.0, ff = 0.0;
  constexpr int RPW = 32 / kRowLanes;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = warp * RPW; base < n; base += nwarps * RPW) {  // warp-uniform bound
    const int64_t i = base + lane / kRowLanes;
    DD sx{0.0, 0.0}, sy{0.0, 0.0};
    if (i < n)
      for (int q = row_ptr[i] + sub; q < row_ptr[i + 1]; q += kRowLanes) {
        double2 a = combine(A, c, q);
        double2 v = xs[col_idx[q]];
        dd_fma(sx, a.x, v.x);
        dd_fma(sx, -a.y, v.y);
        dd_fma(sy, a.x, v.y);
        dd_fma(sy, a.y, v.x);
      }
    sx = row_sum(sx);
    sy = row_sum(sy);
    if (i < n && sub == 0) {
      double2 fi = f[s * n + i];
      double2 ri = make_double2(dd_residual(fi.x, sx), dd_residual(fi.y, sy));
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
    sc->partial[s][blockIdx.x][0] = a;
    sc->partial[s][blockIdx.x][1] = b;
  }
}

__global__ void k_noalloc_norms(NoAllocScratch* sc, int nparts) {
  const int s = blockIdx.x;
  __shared__ double a[256], b[256];
  double x = 0, y = 0;
  for (int q = threadIdx.x; q < nparts; q += blockDim.x) {
    x += sc->partial[s][q][0];
    y += sc->partial[s][q][1];
  }
  a[threadIdx.x] = x;
  b[threadIdx.x] = y;
  __syncthreads();
  for (int o = blockDim.x / 2; o; o >>= 1) {
    if ((int)threadIdx.x < o) { a[threadIdx.x] += a[threadIdx.x + o]; b[threadIdx.x] += b[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) sc->rel[s] = b[0] > 0 ? sqrt(a[0] / b[0]) : sqrt(a[0]);
}

}  // namespace
}  // namespace elp

using namespace elp;

extern "C" int elp_residual_noalloc(elp_model* h, const double* omegas, int n_omega, const double* f_dev,
                                    const double* x_dev, double* r_dev, double* rel_residual_out, void* stream) {
  if (!h || !omegas || !f_dev || !x_dev || !r_dev || !rel_residual_out) {
    set_error("null argument");
    return ELP_ERR_ARG;
  }
  if (n_omega < 1 || n_omega > ELP_NOALLOC_MAX_OMEGA) {
    set_error("n_omega must be between 1 and ELP_NOALLOC_MAX_OMEGA (" + std::to_string(ELP_NOALLOC_MAX_OMEGA) +
              "): the fixed scratch array holds no more frequencies");
    return ELP_ERR_ARG;
  }
  Model& m = h->m;
  if (!m.assembled || !m.dev) { set_error("assemble the model first"); return ELP_ERR_STATE; }
  for (int s = 0; s < n_omega; ++s)
    if (!(omegas[s] > 0.0)) { set_error("angular frequency must be > 0"); return ELP_ERR_ARG; }
  NoAllocScratch* sc = nullptr;
  int rc = scratch_address(&sc);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  Coef coefs[ELP_NOALLOC_MAX_OMEGA];
  for (int s = 0; s < n_omega; ++s) make_coef(m, omegas[s], coefs[s]);
  ELP_CUDA(cudaMemcpyAsync(sc->coef, coefs, sizeof(Coef) * n_omega, cudaMemcpyHostToDevice, st));
  ELP_CUDA(cudaMemsetAsync(sc->rel, 0, sizeof(double) * ELP_NOALLOC_MAX_OMEGA, st));
  const int64_t n = m.n;
  const int nparts = (int)std::min<int64_t>(kNoAllocParts, std::max<int64_t>(1, (n + 255) / 256));
  CombineArgs A = combine_args(m);
  // launched outside the library's launch profiler: its event pairs are
  // created on demand and resolved across every stream, which would break
  // both the no-allocation promise and the independence from other streams
  k_noalloc_residual<<<dim3(nparts, n_omega), 256, 0, st>>>(
      A, sc, m.dev->row_ptr.p, m.dev->col_idx.p, n, reinterpret_cast<const double2*>(x_dev),
      reinterpret_cast<const double2*>(f_dev), reinterpret_cast<double2*>(r_dev));
  k_noalloc_norms<<<n_omega, 256, 0, st>>>(sc, nparts);
  ELP_CUDA(cudaGetLastError());
  ELP_CUDA(cudaMemcpyAsync(rel_residual_out, sc->rel, sizeof(double) * n_omega, cudaMemcpyDeviceToHost, st));
  ELP_CUDA(cudaStreamSynchronize(st));
  return ELP_OK;
}
