// kernels.cuh -- sm_103a kernels of the BSAM adaptive FAS V-cycle (FP64).
//
// Every kernel restates one step of the reference's MATLAB solve path in the
// reference's floating-point operation order (the library is compiled with
// --fmad=false, so no multiply-add is contracted).  Work is flattened per
// level over all patches: a level's items (colour cells, cells, coarse
// cells, ghost items, ...) are numbered consecutively patch after patch and
// cut into 256-item blocks; `blk_p0[b]` names the patch that holds block b's
// first item, `beg[p]..beg[p+1]` the items of patch p.
//
// Memory layout in HBM: one array per field with every patch of every level
// concatenated, each patch column-major (x fastest) like the reference; the
// solution Q and the coarse shadows QC carry their one-cell ghost frame.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "stencil.cuh"

namespace bsam {

// per-patch metadata on the device
struct PatchD {
  int mx, my, par0, level;
  int q_off, c_off, dew_off, dns_off;
  int qc_off, bcg_off, cfd_off, pc_off;
  int win_off, fp_off, corr_off, pad;
  int bc[4];
};

struct Fields {
  double *Q, *F, *QC;
  const double *FTrue, *CC, *ID, *DeW, *DnS, *bcg, *cfd, *pcoef;
  const uint8_t *flags;        // bit0 covered by a finer level, bit1 correction target
  const int *win, *fp;         // window gathers, footprint scatters (2 ints/cell)
};

// one level's work decomposition for one kind of item
struct Decomp {
  const int *beg;              // [np+1] item prefix per patch (level-local)
  const int *blk_p0;           // [nblocks] first patch of each block
  int n, nblocks;
};

struct LevelD {
  const PatchD *patches;       // this level's patches
  double hx, hy, hx2, hy2, ihx2, ihy2;   // ihx2 = 1/hx2 (used only when exact)
};

__device__ __forceinline__ int find_patch(const Decomp &D, int g) {
  int p = __ldg(D.blk_p0 + blockIdx.x);
  while (g >= __ldg(D.beg + p + 1)) ++p;
  return p;
}

// ---------------------------------------------------------------------------
// relax2d (EllipticBSAM/src/ebKernels.m:37-95): one colour of the red-black
// Gauss-Seidel sweep over all patches of a level.  One thread per cell of the
// colour; the partial physical ghosts ((8/3)g + (1/3)u_2 Dirichlet, h g
// Neumann) are formed in registers, the u_1 coupling being folded into
// InvDiagS.  Neighbours of the other colour are not written in this pass,
// so in-place updates equal the reference's candidate-then-write.
template <bool kPow2>
__global__ void __launch_bounds__(kBlock) k_relax(LevelD L, Decomp D, Fields f, int m, double omega) {
  const int g = blockIdx.x * kBlock + threadIdx.x;
  if (g >= D.n) return;
  const int p = find_patch(D, g);
  const PatchD &P = L.patches[p];
  const int mx = P.mx, my = P.my, half = mx >> 1;
  const int s = g - __ldg(D.beg + p);
  const int lj = s / half;
  const int li = 2 * (s - lj * half) + ((m + lj + P.par0) & 1);
  const int ldq = mx + 2;
  double *__restrict__ Q = f.Q + P.q_off;
  const int c = (li + 1) + (lj + 1) * ldq;
  const double *__restrict__ g4 = f.bcg + P.bcg_off;
  double qe = Q[c + 1], qw = Q[c - 1], qn = Q[c + ldq], qs = Q[c - ldq];
  if (li == 0 && P.bc[0]) qw = (P.bc[0] == 1) ? (8.0 / 3.0) * g4[lj] + (1.0 / 3.0) * Q[c + 1] : L.hx * g4[lj];
  if (li == mx - 1 && P.bc[1]) qe = (P.bc[1] == 1) ? (8.0 / 3.0) * g4[my + lj] + (1.0 / 3.0) * Q[c - 1] : L.hx * g4[my + lj];
  if (lj == 0 && P.bc[2]) qs = (P.bc[2] == 1) ? (8.0 / 3.0) * g4[2 * my + li] + (1.0 / 3.0) * Q[c + ldq] : L.hy * g4[2 * my + li];
  if (lj == my - 1 && P.bc[3]) qn = (P.bc[3] == 1) ? (8.0 / 3.0) * g4[2 * my + mx + li] + (1.0 / 3.0) * Q[c - ldq] : L.hy * g4[2 * my + mx + li];
  const double *__restrict__ DeW = f.DeW + P.dew_off;
  const double *__restrict__ DnS = f.DnS + P.dns_off;
  const int cc = P.c_off + li + lj * mx;
  double t = __ldg(f.F + cc);
  t = t + divh<kPow2>(qe * __ldg(DeW + (li + 1) + lj * (mx + 1)), L.hx2, L.ihx2);
  t = t + divh<kPow2>(qw * __ldg(DeW + li + lj * (mx + 1)), L.hx2, L.ihx2);
  t = t + divh<kPow2>(qn * __ldg(DnS + li + (lj + 1) * mx), L.hy2, L.ihy2);
  t = t + divh<kPow2>(qs * __ldg(DnS + li + lj * mx), L.hy2, L.ihy2);
  t = t * __ldg(f.ID + cc);
  Q[c] = (omega == 1.0) ? t : omega * t + (1 - omega) * Q[c];
}

// ---------------------------------------------------------------------------
// Ghost fill (EllipticBSAM/src/ebFillGhosts.m:17-94, ebInterpCf.m:36-154).
// The three ordered stages (coarse-fine interpolation, same-level copy,
// physical closure) are resolved on the host into one final rule per ghost
// cell; every rule reads only interior cells, parent cells or boundary
// data, so a level's ghost cells are filled in one pass.  Physical corners
// read face ghosts and run as a second pass.  Coarse-window values are read
// from the parent's Q directly (the QC ring is refreshed from the same
// cells in the same pass).
enum GhostType : int8_t {
  G_COPY = 0, G_QIF = 1, G_QIF_END = 2, G_LIF = 3, G_LIF_CORNER = 4,
  G_DIRICHLET = 5, G_NEUMANN = 6, G_RING = 7, G_PHYS_CORNER = 8
};

struct GhostItems {
  const int8_t *type;
  const int *dst, *a, *b, *c, *d, *e;
};

__global__ void __launch_bounds__(kBlock) k_ghost(GhostItems G, int off, int n, double *__restrict__ Q,
                                                  double *__restrict__ QC, const double *__restrict__ bcg,
                                                  double hx, double hy) {
  const int t = blockIdx.x * kBlock + threadIdx.x;
  if (t >= n) return;
  const int i = off + t;
  const int8_t ty = G.type[i];
  const int dst = G.dst[i], a = G.a[i];
  constexpr double A1 = -1.0 / 5.0, A2 = 2.0 / 3.0, A3 = 8.0 / 15.0;
  constexpr double B1 = 5.0 / 32.0, B2 = 15.0 / 16.0, B3 = -3.0 / 32.0;
  double v;
  switch (ty) {
    case G_COPY: v = Q[a]; break;
    case G_QIF: v = (A1 * Q[a] + A2 * Q[G.b[i]]) + A3 * Q[G.c[i]]; break;
    case G_QIF_END:
      v = (A1 * Q[a] + A2 * Q[G.b[i]]) + A3 * ((B1 * Q[G.c[i]] + B2 * Q[G.d[i]]) + B3 * Q[G.e[i]]);
      break;
    case G_LIF: v = ((2.0 / 3.0) * Q[G.c[i]] + (2.0 / 3.0) * Q[a]) - (1.0 / 3.0) * Q[G.b[i]]; break;
    case G_LIF_CORNER: v = (2.0 / 3.0) * Q[G.c[i]] + (1.0 / 3.0) * Q[a]; break;
    case G_DIRICHLET: v = ((8.0 / 3.0) * bcg[G.e[i]] - 2 * Q[a]) + (1.0 / 3.0) * Q[G.b[i]]; break;
    case G_NEUMANN: v = Q[a] + (G.b[i] ? hy : hx) * bcg[G.e[i]]; break;
    case G_RING: QC[dst] = Q[a]; return;
    default: v = (Q[a] + Q[G.b[i]]) - Q[G.c[i]]; break;  // G_PHYS_CORNER
  }
  Q[dst] = v;
}

// ---------------------------------------------------------------------------
// restrict2 (ebKernels.m:98-102) of each patch interior into its QC interior
// and, for 'restrict' (ebTransfer.m:10-33), into the parent's Q over the
// footprint.  One thread per coarse cell.
__global__ void __launch_bounds__(kBlock) k_restrict(LevelD L, Decomp D, Fields f, int to_parent) {
  const int g = blockIdx.x * kBlock + threadIdx.x;
  if (g >= D.n) return;
  const int p = find_patch(D, g);
  const PatchD &P = L.patches[p];
  const int cmx = P.mx >> 1;
  const int s = g - __ldg(D.beg + p);
  const int cj = s / cmx, ci = s - cj * cmx;
  const int ldq = P.mx + 2;
  const double *__restrict__ Q = f.Q + P.q_off;
  const int c = (2 * ci + 1) + (2 * cj + 1) * ldq;
  const double R = 0.25 * (((Q[c] + Q[c + 1]) + Q[c + ldq]) + Q[c + ldq + 1]);
  f.QC[P.qc_off + (ci + 1) + (cj + 1) * (cmx + 2)] = R;
  if (to_parent) f.Q[__ldg(f.fp + 2 * (P.fp_off + s))] = R;
}

// QC ring <- parent Q (ebTransfer.m:35-55 'ring'), one thread per ring cell
__global__ void __launch_bounds__(kBlock) k_ring(const int *__restrict__ ring, int off, int n, const double *Q,
                                                 double *__restrict__ QC) {
  const int t = blockIdx.x * kBlock + threadIdx.x;
  if (t >= n) return;
  const int i = off + t;
  QC[__ldg(ring + 2 * i + 1)] = Q[__ldg(ring + 2 * i)];
}

// ---------------------------------------------------------------------------
// FAS coarse load over the footprint (ebCoarseLoad.m:17-32 with
// ebParentCoeffs.m): F_parent = restrict2(F - op(Q)) + op_c(QC, parent coeffs).
// One thread per coarse cell; the four fine residuals are summed in the
// restrict2 order (1,1), (2,1), (1,2), (2,2).
template <bool kPow2>
__global__ void __launch_bounds__(kBlock) k_coarse_load(LevelD L, LevelD Lc, Decomp D, Fields f) {
  const int g = blockIdx.x * kBlock + threadIdx.x;
  if (g >= D.n) return;
  const int p = find_patch(D, g);
  const PatchD &P = L.patches[p];
  const int mx = P.mx, cmx = mx >> 1, cmy = P.my >> 1;
  const int s = g - __ldg(D.beg + p);
  const int cj = s / cmx, ci = s - cj * cmx;
  const double *Qp = f.Q + P.q_off;
  const double *DeW = f.DeW + P.dew_off, *DnS = f.DnS + P.dns_off;
  const double *Fp = f.F + P.c_off, *CC = f.CC + P.c_off;
  double rf[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int li = 2 * ci + (t & 1), lj = 2 * cj + (t >> 1);
    const int cc = li + lj * mx;
    rf[t] = Fp[cc] - op_cell<kPow2>(Qp, mx + 2, DeW, DnS, CC[cc], mx, li, lj, L.hx2, L.hy2, L.ihx2, L.ihy2);
  }
  const double rr = 0.25 * (((rf[0] + rf[1]) + rf[2]) + rf[3]);
  const double *PDeW = f.pcoef + P.pc_off;
  const double *PDnS = PDeW + (cmx + 1) * cmy;
  const double *PCC = PDnS + cmx * (cmy + 1);
  const double lc = op_cell<kPow2>(f.QC + P.qc_off, cmx + 2, PDeW, PDnS, PCC[s], cmx, ci, cj, Lc.hx2, Lc.hy2,
                                   Lc.ihx2, Lc.ihy2);
  f.F[__ldg(f.fp + 2 * (P.fp_off + s) + 1)] = rr + lc;
}

// ebFaceCorrections (ebFaceCorrections.m:18-61): correction of coarse face j
// on face fc (0 W, 1 E, 2 S, 3 N) of patch P; hc2 is the parent h^2 in the
// face-normal direction
template <bool kPow2>
__device__ __forceinline__ double face_corr(const PatchD &P, const Fields &f, int fc, int j, double hc2,
                                            double ihc2) {
  const int mx = P.mx, my = P.my, cmx = mx >> 1, cmy = my >> 1;
  const int ldq = mx + 2, ldc = cmx + 2;
  const double *Q = f.Q + P.q_off, *QC = f.QC + P.qc_off;
  const double *DeW = f.DeW + P.dew_off, *DnS = f.DnS + P.dns_off, *cfd = f.cfd + P.cfd_off;
  // 0-based padded indices; fine rows 2j+1, 2j+2 of the padded array
  double v;
  switch (fc) {
    case 0: {
      const int r1 = 2 * j + 1, r2 = 2 * j + 2;
      v = (DeW[(2 * j) * (mx + 1)] * (Q[1 + r1 * ldq] - Q[r1 * ldq]) +
           DeW[(2 * j + 1) * (mx + 1)] * (Q[1 + r2 * ldq] - Q[r2 * ldq])) +
          cfd[j] * (QC[(j + 1) * ldc] - QC[1 + (j + 1) * ldc]);
      break;
    }
    case 1: {
      const int r1 = 2 * j + 1, r2 = 2 * j + 2;
      v = (DeW[mx + (2 * j) * (mx + 1)] * (Q[mx + r1 * ldq] - Q[mx + 1 + r1 * ldq]) +
           DeW[mx + (2 * j + 1) * (mx + 1)] * (Q[mx + r2 * ldq] - Q[mx + 1 + r2 * ldq])) +
          cfd[cmy + j] * (QC[cmx + 1 + (j + 1) * ldc] - QC[cmx + (j + 1) * ldc]);
      break;
    }
    case 2: {
      const int c1 = 2 * j + 1, c2 = 2 * j + 2;
      v = (DnS[2 * j] * (Q[c1 + ldq] - Q[c1]) + DnS[2 * j + 1] * (Q[c2 + ldq] - Q[c2])) +
          cfd[2 * cmy + j] * (QC[j + 1] - QC[j + 1 + ldc]);
      break;
    }
    default: {
      const int c1 = 2 * j + 1, c2 = 2 * j + 2;
      v = (DnS[2 * j + my * mx] * (Q[c1 + my * ldq] - Q[c1 + (my + 1) * ldq]) +
           DnS[2 * j + 1 + my * mx] * (Q[c2 + my * ldq] - Q[c2 + (my + 1) * ldq])) +
          cfd[2 * cmy + cmx + j] * (QC[j + 1 + (cmy + 1) * ldc] - QC[j + 1 + cmy * ldc]);
      break;
    }
  }
  return divh<kPow2>(v, hc2, ihc2);
}

// Flux-balance corrections (ebCoarseLoad.m:37-45) in gather form: one thread
// per target coarse cell adds its corrections in the reference's order
// (fine patch ascending, faces W, E, S, N).  `items` encode
// (level-local patch << 2 | face) and `jj` the coarse face index.
template <bool kPow2>
__global__ void __launch_bounds__(kBlock) k_corr(LevelD L, LevelD Lc, Fields f, const int *__restrict__ tcell,
                                                 const int *__restrict__ tbeg, const int *__restrict__ items,
                                                 const int *__restrict__ jj, int n) {
  const int t = blockIdx.x * kBlock + threadIdx.x;
  if (t >= n) return;
  const int cell = tcell[t];
  double v = f.F[cell];
  for (int i = tbeg[t]; i < tbeg[t + 1]; ++i) {
    const int it = items[i];
    const int fc = it & 3;
    const PatchD &P = L.patches[it >> 2];
    v = v + face_corr<kPow2>(P, f, fc, jj[i], fc < 2 ? Lc.hx2 : Lc.hy2, fc < 2 ? Lc.ihx2 : Lc.ihy2);
  }
  f.F[cell] = v;
}

// ---------------------------------------------------------------------------
// prolongBilin (ebKernels.m:105-123) of the parent window: 'correct'
// (ebTransfer.m:57-71) adds P(W - QC) to the interior; mode 0 writes P(W)
// (new-level initial guess, ebAddLevel.m:26-31).  One thread per coarse cell
// writes its four fine cells.
__global__ void __launch_bounds__(kBlock) k_prolong(LevelD L, Decomp D, Fields f, int correct) {
  const int g = blockIdx.x * kBlock + threadIdx.x;
  if (g >= D.n) return;
  const int p = find_patch(D, g);
  const PatchD &P = L.patches[p];
  const int cm = P.mx >> 1;
  const int s = g - __ldg(D.beg + p);
  const int b = s / cm, a = s - b * cm;
  const int ldw = cm + 2;
  const int *win = f.win + P.win_off;
  const double *QC = f.QC + P.qc_off;
  double E[3][3];
#pragma unroll
  for (int dj = 0; dj < 3; ++dj)
#pragma unroll
    for (int di = 0; di < 3; ++di) {
      const int w = (a + di) + (b + dj) * ldw;
      const double wv = f.Q[__ldg(win + w)];
      E[dj][di] = correct ? wv - QC[w] : wv;
    }
  const double C = E[1][1], Wm = E[1][0], Wp = E[1][2], Sm = E[0][1], Sp = E[2][1];
  const double f11 = (((9 * C + 3 * Wm) + 3 * Sm) + E[0][0]) / 16;
  const double f21 = (((9 * C + 3 * Wp) + 3 * Sm) + E[0][2]) / 16;
  const double f12 = (((9 * C + 3 * Wm) + 3 * Sp) + E[2][0]) / 16;
  const double f22 = (((9 * C + 3 * Wp) + 3 * Sp) + E[2][2]) / 16;
  const int ldq = P.mx + 2;
  double *Q = f.Q + P.q_off;
  const int c = (2 * a + 1) + (2 * b + 1) * ldq;
  if (correct) {
    Q[c] = Q[c] + f11;
    Q[c + 1] = Q[c + 1] + f21;
    Q[c + ldq] = Q[c + ldq] + f12;
    Q[c + ldq + 1] = Q[c + ldq + 1] + f22;
  } else {
    Q[c] = f11;
    Q[c + 1] = f21;
    Q[c + ldq] = f12;
    Q[c + ldq + 1] = f22;
  }
}

// ---------------------------------------------------------------------------
// Coarsest solve (ebCoarsest.m:79-91): u = Ainv (F + bcRhs), one warp per
// row; lane l sums columns l, l+32, ... in order, then a halving tree.
__global__ void __launch_bounds__(kBlock) k_coarsest(const double *__restrict__ Ainv, const double *__restrict__ bcRhs,
                                                     Fields f, int c_off, int q_off, int n1, int N) {
  const int row = (blockIdx.x * kBlock + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= N) return;
  const double *a = Ainv + (size_t)row * N;
  const double *F = f.F + c_off;
  double s = 0.0;
  for (int c = lane; c < N; c += 32) s = s + a[c] * (F[c] + bcRhs[c]);
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    const double o = __shfl_down_sync(0xffffffffu, s, off);
    if (lane < off) s = s + o;
  }
  if (lane == 0) {
    const int i = row % n1, j = row / n1;
    f.Q[q_off + (i + 1) + (j + 1) * (n1 + 2)] = s;
  }
}

// ---------------------------------------------------------------------------
// Composite residual (ebCompResidual.m:54-83): r = FTrue - op(Q) on visible
// cells; correction targets are skipped here and handled by
// k_residual_targets.  Max-norms reduce through an order-free atomic max on
// the bit pattern of non-negative doubles; the L2 sum keeps one partial per
// block in a fixed slot.
struct ResAcc {
  unsigned long long linf_bits, fnorm_bits;
  double out[5];        // linf, l2, fnorm, rel, ncell
};

__device__ __forceinline__ void block_reduce_store(double li, double sq, double fn, ResAcc *acc, double *slot) {
  __shared__ double s_li[kBlock / 32], s_sq[kBlock / 32], s_fn[kBlock / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    li = fmax(li, __shfl_down_sync(0xffffffffu, li, off));
    fn = fmax(fn, __shfl_down_sync(0xffffffffu, fn, off));
    sq = sq + __shfl_down_sync(0xffffffffu, sq, off);
  }
  if (lane == 0) { s_li[w] = li; s_sq[w] = sq; s_fn[w] = fn; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double L = s_li[0], S = s_sq[0], Fn = s_fn[0];
    for (int i = 1; i < kBlock / 32; ++i) { L = fmax(L, s_li[i]); S = S + s_sq[i]; Fn = fmax(Fn, s_fn[i]); }
    atomicMax(&acc->linf_bits, (unsigned long long)__double_as_longlong(L));
    atomicMax(&acc->fnorm_bits, (unsigned long long)__double_as_longlong(Fn));
    *slot = S;
  }
}

template <bool kPow2>
__global__ void __launch_bounds__(kBlock) k_residual(LevelD L, Decomp D, Fields f, ResAcc *acc, double *slots,
                                                     int skip_targets) {
  const int g = blockIdx.x * kBlock + threadIdx.x;
  double li = 0, sq = 0, fn = 0;
  if (g < D.n) {
    const int p = find_patch(D, g);
    const PatchD &P = L.patches[p];
    const int mx = P.mx;
    const int s = g - __ldg(D.beg + p);
    const int lj = s / mx, lx = s - lj * mx;
    const int cc = P.c_off + s;
    const uint8_t fl = f.flags[cc];
    // covered cells are not part of the composite norm; correction targets
    // are evaluated by k_residual_targets when the corrections are on
    if (!(fl & 1) && !(skip_targets && (fl & 2))) {
      const double ft = f.FTrue[cc];
      const double r = ft - op_cell<kPow2>(f.Q + P.q_off, mx + 2, f.DeW + P.dew_off, f.DnS + P.dns_off, f.CC[cc],
                                           mx, lx, lj, L.hx2, L.hy2, L.ihx2, L.ihy2);
      li = fabs(r);
      sq = r * r;
      fn = fabs(ft);
    }
  }
  block_reduce_store(li, sq, fn, acc, slots + blockIdx.x);
}

// residual at correction targets of level k-1 (they are visible cells):
// r = FTrue - op(Q) + corrections in order
template <bool kPow2>
__global__ void __launch_bounds__(kBlock) k_residual_targets(LevelD Lf, LevelD Lc, const PatchD *patches_c, Fields f,
                                                             const int *__restrict__ tcell, const int *__restrict__ tpatch,
                                                             const int *__restrict__ tbeg, const int *__restrict__ items,
                                                             const int *__restrict__ jj, int n, ResAcc *acc,
                                                             double *slots) {
  const int t = blockIdx.x * kBlock + threadIdx.x;
  double li = 0, sq = 0, fn = 0;
  if (t < n) {
    const int cell = tcell[t];
    const PatchD &Pc = patches_c[tpatch[t]];
    const int s = cell - Pc.c_off;
    const int lj = s / Pc.mx, lx = s - lj * Pc.mx;
    const double ft = f.FTrue[cell];
    double r = ft - op_cell<kPow2>(f.Q + Pc.q_off, Pc.mx + 2, f.DeW + Pc.dew_off, f.DnS + Pc.dns_off, f.CC[cell],
                                   Pc.mx, lx, lj, Lc.hx2, Lc.hy2, Lc.ihx2, Lc.ihy2);
    for (int i = tbeg[t]; i < tbeg[t + 1]; ++i) {
      const int it = items[i];
      const int fc = it & 3;
      r = r + face_corr<kPow2>(Lf.patches[it >> 2], f, fc, jj[i], fc < 2 ? Lc.hx2 : Lc.hy2,
                               fc < 2 ? Lc.ihx2 : Lc.ihy2);
    }
    if (!(f.flags[cell] & 1)) {
      li = fabs(r);
      sq = r * r;
      fn = fabs(ft);
    }
  }
  block_reduce_store(li, sq, fn, acc, slots + blockIdx.x);
}

// finish the residual: L2 from the per-block partials in slot order, each
// level's partials weighted by its cell area; rel = linf / max(fnorm, realmin)
__global__ void k_residual_final(ResAcc *acc, const double *slots, const int *level_slot0, const double *area,
                                 int nlevels_res, double ncell) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double l2sq = 0;
  for (int l = 0; l < nlevels_res; ++l) {
    double s = 0;
    for (int i = level_slot0[l]; i < level_slot0[l + 1]; ++i) s = s + slots[i];
    l2sq = l2sq + s * area[l];
  }
  const double linf = __longlong_as_double((long long)acc->linf_bits);
  double fnorm = __longlong_as_double((long long)acc->fnorm_bits);
  fnorm = fnorm > 2.2250738585072014e-308 ? fnorm : 2.2250738585072014e-308;
  acc->out[0] = linf;
  acc->out[1] = sqrt(l2sq);
  acc->out[2] = fnorm;
  acc->out[3] = linf / fnorm;
  acc->out[4] = ncell;
  acc->linf_bits = 0;
  acc->fnorm_bits = 0;
}

// ---------------------------------------------------------------------------
// Composite sums over visible cells (ebCompositeMean.m, ebMassCheck.m lhs):
// per-block partials of sum(u), sum(C u - FTrue), sum(|FTrue|)
__global__ void __launch_bounds__(kBlock) k_sums(LevelD L, Decomp D, Fields f, double *partials) {
  const int g = blockIdx.x * kBlock + threadIdx.x;
  double su = 0, sm = 0, sa = 0, nv = 0;
  if (g < D.n) {
    const int p = find_patch(D, g);
    const PatchD &P = L.patches[p];
    const int s = g - __ldg(D.beg + p);
    const int lj = s / P.mx, lx = s - lj * P.mx;
    const int cc = P.c_off + s;
    if (!(f.flags[cc] & 1)) {
      const double u = f.Q[P.q_off + (lx + 1) + (lj + 1) * (P.mx + 2)];
      su = u;
      sm = f.CC[cc] * u - f.FTrue[cc];
      sa = fabs(f.FTrue[cc]);
      nv = 1;
    }
  }
  __shared__ double sh[4][kBlock];
  sh[0][threadIdx.x] = su; sh[1][threadIdx.x] = sm; sh[2][threadIdx.x] = sa; sh[3][threadIdx.x] = nv;
  __syncthreads();
  for (int off = kBlock / 2; off >= 1; off >>= 1) {
    if (threadIdx.x < off)
      for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] = sh[q][threadIdx.x] + sh[q][threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 4; ++q) partials[4 * blockIdx.x + q] = sh[q][0];
}

}  // namespace bsam
