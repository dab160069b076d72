// bsam_geom.cu -- device part of the diffuse-domain coefficient sampling:
// the squared distance from sample points to a closed polygon
// (DiffuseDomainBSAM/src/ddStarfishGeometry.m:140-177, exact point-to-
// segment distance).  The host keeps the O(n) parts (the radial sign test
// and the starting candidate, which need atan2/cos/sin); the device does the
// O(n x segments) minimum.  Per segment the arithmetic is the reference's
//   t  = ((x - ax) ex + (y - ay) ey) / |e|^2,  t = max(0, min(1, t))
//   dd = ((x - ax) - t ex)^2 + ((y - ay) - t ey)^2
// in that order (no contraction), and a minimum does not depend on the
// order of its terms, so the result equals the host's bit for bit.
// Segments are pruned in groups of eight by the distance to the group's
// bounding box with the host's slack (a group is evaluated unless its box is
// farther than best + 64 eps), which never drops the minimising segment.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>
#include <string>

#include "bsam_dev.h"
#include "internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kGroup = 8;               // segments per pruning box
constexpr int kTile = 1024;             // segments staged in shared memory per pass

struct SegTile {
  double ax[kTile], ay[kTile], ex[kTile], ey[kTile], l2[kTile];
  double box[kTile / kGroup][4];        // minx miny maxx maxy
};

__global__ void __launch_bounds__(kThreads) k_segdist(const double *__restrict__ v, int ns,
                                                      const double *__restrict__ x, const double *__restrict__ y,
                                                      double *__restrict__ best, int64_t n) {
  extern __shared__ __align__(16) unsigned char smem[];
  SegTile &T = *reinterpret_cast<SegTile *>(smem);
  const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const bool on = i < n;
  const double px = on ? x[i] : 0.0, py = on ? y[i] : 0.0;
  double b = on ? best[i] : 0.0;
  for (int s0 = 0; s0 < ns; s0 += kTile) {
    const int nt = min(kTile, ns - s0);
    __syncthreads();
    for (int j = threadIdx.x; j < nt; j += kThreads) {
      const int g = s0 + j;
      const double ax = v[2 * g], ay = v[2 * g + 1];
      const double ex = v[2 * (g + 1)] - ax, ey = v[2 * (g + 1) + 1] - ay;
      T.ax[j] = ax;
      T.ay[j] = ay;
      T.ex[j] = ex;
      T.ey[j] = ey;
      T.l2[j] = ex * ex + ey * ey;
    }
    for (int q = threadIdx.x; q < (nt + kGroup - 1) / kGroup; q += kThreads) {
      // box over the group's vertices v(g .. g+len), as the host builds it
      const int g0 = s0 + q * kGroup, g1 = min(s0 + nt, g0 + kGroup);
      double mnx = v[2 * g0], mny = v[2 * g0 + 1], mxx = mnx, mxy = mny;
      for (int g = g0 + 1; g <= g1; ++g) {
        mnx = fmin(mnx, v[2 * g]);
        mxx = fmax(mxx, v[2 * g]);
        mny = fmin(mny, v[2 * g + 1]);
        mxy = fmax(mxy, v[2 * g + 1]);
      }
      T.box[q][0] = mnx;
      T.box[q][1] = mny;
      T.box[q][2] = mxx;
      T.box[q][3] = mxy;
    }
    __syncthreads();
    if (!on) continue;
    const int ng = (nt + kGroup - 1) / kGroup;
    for (int q = 0; q < ng; ++q) {
      const double dx = fmax(fmax(T.box[q][0] - px, 0.0), px - T.box[q][2]);
      const double dy = fmax(fmax(T.box[q][1] - py, 0.0), py - T.box[q][3]);
      if (!(dx * dx + dy * dy <= b + 64 * DBL_EPSILON)) continue;
      const int j1 = min(nt, (q + 1) * kGroup);
      for (int j = q * kGroup; j < j1; ++j) {
        const double rx = px - T.ax[j], ry = py - T.ay[j];
        double t = (rx * T.ex[j] + ry * T.ey[j]) / T.l2[j];
        t = fmax(0.0, fmin(1.0, t));
        const double qx = rx - t * T.ex[j], qy = ry - t * T.ey[j];
        b = fmin(b, qx * qx + qy * qy);
      }
    }
  }
  if (on) best[i] = b;
}

int gfail(int code, const std::string &m) { return bsam_internal_set_error(code, m); }

#define GCK(x)                                                                                      \
  do {                                                                                              \
    cudaError_t e_ = (x);                                                                           \
    if (e_ != cudaSuccess)                                                                          \
      return gfail(e_ == cudaErrorMemoryAllocation ? BSAM_ERR_NOMEM : BSAM_ERR_CUDA,                 \
                   std::string(#x) + ": " + cudaGetErrorString(e_));                                \
  } while (0)

}  // namespace

extern "C" int bsam_polygon_dist2(bsam_ctx ctx, const double *verts, int nverts, const double *x, const double *y,
                                  double *best, int64_t n) {
  if (!ctx || !verts || nverts < 2 || n < 0 || (n && (!x || !y || !best)))
    return gfail(BSAM_ERR_ARG, "bsam_polygon_dist2: bad argument");
  if (n == 0) return BSAM_OK;
  GCK(cudaSetDevice(ctx->device));
  const size_t nv = 2 * (size_t)nverts;
  const size_t need = sizeof(double) * (nv + 3 * (size_t)n);
  if (need > ctx->scratch_bytes) {   // stream-ordered: no device-wide synchronisation
    if (ctx->scratch) cudaFreeAsync(ctx->scratch, ctx->stream);
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
    GCK(cudaMallocAsync(&ctx->scratch, need, ctx->stream));
    ctx->scratch_bytes = need;
  }
  double *dv = (double *)ctx->scratch, *dx = dv + nv, *dy = dx + n, *db = dy + n;
  cudaStream_t s = ctx->stream;
  GCK(cudaMemcpyAsync(dv, verts, sizeof(double) * nv, cudaMemcpyHostToDevice, s));
  GCK(cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  GCK(cudaMemcpyAsync(dy, y, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  GCK(cudaMemcpyAsync(db, best, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  const size_t shm = sizeof(SegTile);
  static thread_local int attr_device = -1;
  if (attr_device != ctx->device) {
    GCK(cudaFuncSetAttribute(k_segdist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
    attr_device = ctx->device;
  }
  const unsigned grid = (unsigned)((n + kThreads - 1) / kThreads);
  k_segdist<<<grid, kThreads, shm, s>>>(dv, nverts - 1, dx, dy, db, n);
  GCK(cudaGetLastError());
  GCK(cudaMemcpyAsync(best, db, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  GCK(cudaStreamSynchronize(s));
  return BSAM_OK;
}
