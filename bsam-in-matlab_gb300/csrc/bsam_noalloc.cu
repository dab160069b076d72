// bsam_noalloc.cu -- a residual-norm entry point that allocates nothing.
//
// Some callers cannot call cudaMalloc: a host that hands the library memory
// from its own pool (a MATLAB gpuArray, a framework's caching allocator), or
// code that must not allocate while it runs.  bsam_patch_residual_noalloc
// evaluates the plain residual norms of one patch on caller-owned device
// arrays: r = FTrue - op2d(Q) (ebKernels.m:13-25) over the cells whose
// `covered` byte is 0, with linf, l2, fnorm and rel formed as in
// ebCompResidual.m:66-83.  It adds no coarse-fine flux corrections
// (ebCompResidual.m:40-65), so it equals the reference's composite residual
// only for a patch that no finer level touches.  Its block-reduction scratch
// is the file-scope device array below, so the call performs no device
// allocation of any kind.
//
// The scratch is a static __device__ array of BSAM_NOALLOC_MAX_BLOCKS + 4
// doubles (16388 * 8 B = 128 KiB); every GPU that loads the library holds it
// until the process exits.  All calls share it and it keeps the last call's
// contents, so the accumulators are cleared at the start of every call, and
// calls that overlap on the GPU (different streams or host threads) race on
// it and must be serialised by the caller.
//
// Host code must not pass the array's name to a kernel: on the host the
// symbol is a stand-in, not a device address.  Every call looks the device
// address up with cudaGetSymbolAddress for the current device (a host-side
// lookup that enqueues no work), so the address stays right after a device
// reset, which reloads the library's device code in a new context.  The
// first call on a device may load that code; make it before any stream
// capture.
#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "bsam_dev.h"
#include "stencil.cuh"

// records the message returned by bsam_last_error() (defined in bsam_dev.cu)
int bsam_internal_set_error(int code, const std::string &msg);

namespace {

constexpr int kMaxBlocks = BSAM_NOALLOC_MAX_BLOCKS;

// [0..kMaxBlocks) per-block L2 partials; [kMaxBlocks] linf bits,
// [kMaxBlocks+1] fnorm bits, [kMaxBlocks+2] visible-cell count
static __device__ __align__(256) double g_noalloc_scratch[kMaxBlocks + 4];

__global__ void k_noalloc_clear(double *scratch) {
  unsigned long long *w = reinterpret_cast<unsigned long long *>(scratch + kMaxBlocks);
  if (threadIdx.x < 3) w[threadIdx.x] = 0ull;
}

template <bool kPow2>
__global__ void __launch_bounds__(bsam::kBlock) k_noalloc_residual(const double *__restrict__ Q,
                                                                  const double *__restrict__ FTrue,
                                                                  const double *__restrict__ DeW,
                                                                  const double *__restrict__ DnS,
                                                                  const double *__restrict__ CC,
                                                                  const uint8_t *__restrict__ covered, int mx, int my,
                                                                  double hx2, double hy2, double ihx2, double ihy2,
                                                                  double *scratch) {
  const int g = blockIdx.x * bsam::kBlock + threadIdx.x;
  double li = 0, sq = 0, fn = 0, nv = 0;
  if (g < mx * my && !(covered && covered[g])) {
    const int lj = g / mx, lx = g - lj * mx;
    const double ft = FTrue[g];
    const double r = ft - bsam::op_cell<kPow2>(Q, mx + 2, DeW, DnS, CC[g], mx, lx, lj, hx2, hy2, ihx2, ihy2);
    li = fabs(r);
    sq = r * r;
    fn = fabs(ft);
    nv = 1;
  }
  __shared__ double s_li[bsam::kBlock / 32], s_sq[bsam::kBlock / 32], s_fn[bsam::kBlock / 32],
      s_nv[bsam::kBlock / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    li = fmax(li, __shfl_down_sync(0xffffffffu, li, off));
    fn = fmax(fn, __shfl_down_sync(0xffffffffu, fn, off));
    sq = sq + __shfl_down_sync(0xffffffffu, sq, off);
    nv = nv + __shfl_down_sync(0xffffffffu, nv, off);
  }
  if (lane == 0) { s_li[w] = li; s_sq[w] = sq; s_fn[w] = fn; s_nv[w] = nv; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double L = s_li[0], S = s_sq[0], Fn = s_fn[0], N = s_nv[0];
    for (int i = 1; i < bsam::kBlock / 32; ++i) {
      L = fmax(L, s_li[i]);
      S = S + s_sq[i];
      Fn = fmax(Fn, s_fn[i]);
      N = N + s_nv[i];
    }
    // fmax drops a NaN operand, so L (Fn) is NaN only when every value of
    // the block was; a NaN then counts as 0, like MATLAB's max, which
    // ignores NaN (the bit-pattern maximum below would otherwise rank it
    // above +Inf)
    if (!(L >= 0.0)) L = 0.0;
    if (!(Fn >= 0.0)) Fn = 0.0;
    unsigned long long *acc = reinterpret_cast<unsigned long long *>(scratch + kMaxBlocks);
    atomicMax(acc + 0, (unsigned long long)__double_as_longlong(L));
    atomicMax(acc + 1, (unsigned long long)__double_as_longlong(Fn));
    atomicAdd(acc + 2, (unsigned long long)N);
    scratch[blockIdx.x] = S;
  }
}

// out = {linf, l2, fnorm, rel, ncell}; L2 sums the block partials in order
__global__ void k_noalloc_final(const double *scratch, int nblocks, double area, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0;
  for (int i = 0; i < nblocks; ++i) s = s + scratch[i];
  const unsigned long long *acc = reinterpret_cast<const unsigned long long *>(scratch + kMaxBlocks);
  const double linf = __longlong_as_double((long long)acc[0]);
  double fnorm = __longlong_as_double((long long)acc[1]);
  fnorm = fnorm > 2.2250738585072014e-308 ? fnorm : 2.2250738585072014e-308;
  out[0] = linf;
  out[1] = sqrt(s * area);
  out[2] = fnorm;
  out[3] = linf / fnorm;
  out[4] = (double)acc[2];
}

int nerr(int code, const std::string &m) { return bsam_internal_set_error(code, m); }

bool pow2(double x) {
  int e;
  return x > 0 && std::frexp(x, &e) == 0.5;
}

// device address of the scratch array on the current device, looked up on
// every call (the address belongs to the device's current context)
int scratch_for_current_device(double **out) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return nerr(BSAM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  *out = static_cast<double *>(p);
  return BSAM_OK;
}

}  // namespace

extern "C" int bsam_patch_residual_noalloc(const double *Q, const double *FTrue, const double *DeW, const double *DnS,
                                           const double *CC, const uint8_t *covered, int mx, int my, double hx,
                                           double hy, double *out, void *stream) {
  if (!Q || !FTrue || !DeW || !DnS || !CC || !out) return nerr(BSAM_ERR_ARG, "null device pointer");
  if (mx < 1 || my < 1 || !(hx > 0) || !(hy > 0)) return nerr(BSAM_ERR_ARG, "invalid patch size or spacing");
  const long long cells = (long long)mx * my;
  const long long nb = (cells + bsam::kBlock - 1) / bsam::kBlock;
  if (nb > kMaxBlocks)
    return nerr(BSAM_ERR_ARG, "patch of " + std::to_string(cells) + " cells exceeds the no-allocation limit of " +
                                  std::to_string((long long)kMaxBlocks * bsam::kBlock) + " cells");
  double *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const double hx2 = hx * hx, hy2 = hy * hy;
  k_noalloc_clear<<<1, 32, 0, s>>>(scratch);
  if (pow2(hx2) && pow2(hy2))
    k_noalloc_residual<true><<<(int)nb, bsam::kBlock, 0, s>>>(Q, FTrue, DeW, DnS, CC, covered, mx, my, hx2, hy2,
                                                               1.0 / hx2, 1.0 / hy2, scratch);
  else
    k_noalloc_residual<false><<<(int)nb, bsam::kBlock, 0, s>>>(Q, FTrue, DeW, DnS, CC, covered, mx, my, hx2, hy2,
                                                                1.0 / hx2, 1.0 / hy2, scratch);
  k_noalloc_final<<<1, 32, 0, s>>>(scratch, (int)nb, hx * hy, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return nerr(BSAM_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return BSAM_OK;
}
