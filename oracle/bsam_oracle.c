/*
 * bsam_oracle.c -- CPU oracle for the BSAM adaptive FAS V-cycle solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker: a plain-C
 * restatement of the reference's MATLAB solve path, in the reference's
 * floating-point operation order (compile with -ffp-contract=off, no fast
 * math), operating on the same flat patch-descriptor tables that the CUDA
 * library receives.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it; the product path never does.
 *
 * Every routine cites the reference function it restates (paths relative
 * to the BSAM-in-MATLAB repository).  The structure follows the reference
 * literally: per-patch loops, the three ordered ghost-fill stages, the
 * strided colour pass that writes one colour of candidates, the scatter of
 * the FAS coarse load followed by the ordered flux-correction adds.
 *
 * The one place the reference is not reproducible bitwise is its sparse LU
 * coarsest solve (MATLAB `decomposition`); here, as on the device, the
 * coarsest solve is one dense product with the host-computed inverse in a
 * fixed summation order (32 strided partial sums, then a halving tree).
 *
 * Parallelism: OpenMP over the patches of a level inside each stage (the
 * stages are independent per patch in the reference too); every ordered
 * reduction keeps a fixed order, so results do not depend on the thread
 * count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

/* per-level descriptor columns (bsam/flat.py LD_*) */
enum { LD_N0, LD_N1, LD_P0, LD_P1, LD_CELL0, LD_CELL1, LD_Q0, LD_Q1, LD };
/* per-patch descriptor columns (bsam/flat.py PD_*) */
enum {
  PD_LEVEL, PD_ILO, PD_IHI, PD_JLO, PD_JHI, PD_MX, PD_MY, PD_PAR0,
  PD_BCW, PD_BCE, PD_BCS, PD_BCN, PD_FIW, PD_FIE, PD_FIS, PD_FIN,
  PD_CCSW, PD_CCSE, PD_CCNW, PD_CCNE,
  PD_QOFF, PD_COFF, PD_DEWOFF, PD_DNSOFF, PD_QCOFF, PD_BCGOFF, PD_CFDOFF, PD_PCOFF,
  PD_SAME0, PD_SAME1, PD_RING0, PD_RING1, PD_WIN0, PD_FP0, PD_CORR0, PD_PARENT, PD
};

typedef struct {
  int nlev, root_idx, npatch;
  const int32_t *levels;
  const double *hs;
  const int32_t *patches;
  double *Q, *F, *FTrue, *QC;
  const double *CC, *ID, *DeW, *DnS, *bcg, *cfd, *pcoef;
  const uint8_t *covered;
  const int32_t *same, *ring, *win, *fp, *corr;
  const double *Ainv, *bcRhs;
  int ncoarse;
  /* options (ebOptions) */
  int npre, npost, qif, mass_corr, max_vcycles;
  double omega, rel_tol;
} OHier;

typedef struct { double linf, l2, fnorm, rel; long long ncell; } ORes;

#define PR(p) (h->patches + (size_t)(p) * PD)
/* padded Q of patch p, 1-based (i, j) like MATLAB */
#define QP(r, i, j) h->Q[(r)[PD_QOFF] + ((i) - 1) + (size_t)((j) - 1) * ((r)[PD_MX] + 2)]
#define QCP(r, i, j) h->QC[(r)[PD_QCOFF] + ((i) - 1) + (size_t)((j) - 1) * ((r)[PD_MX] / 2 + 2)]

static const double A1 = -1.0 / 5.0, A2 = 2.0 / 3.0, A3 = 8.0 / 15.0;
static const double B1 = 5.0 / 32.0, B2 = 15.0 / 16.0, B3 = -3.0 / 32.0;

/* ---------------------------------------------------------------------- */
/* ebInterpCf (EllipticBSAM/src/ebInterpCf.m:36-154) for one patch          */
static void interp_cf(OHier *h, const int32_t *r) {
  const int mx = r[PD_MX], my = r[PD_MY], cmx = mx / 2, cmy = my / 2;
  const int qif = h->qif;
  const int32_t *fint = r + PD_FIW;
  int cCF[4];
  for (int c = 0; c < 4; ++c) cCF[c] = (r[PD_CCSW + c] == 3);
#define Q(i, j) QP(r, i, j)
#define QC(i, j) QCP(r, i, j)
  if (fint[0]) {  /* WEST */
    if (qif) {
      for (int rho = 3; rho <= my - 1; rho += 2) Q(1, rho) = A1 * Q(3, rho + 2) + A2 * Q(2, rho + 1) + A3 * QC(1, (rho + 1) / 2);
      for (int rho = 4; rho <= my; rho += 2) Q(1, rho) = A1 * Q(3, rho - 2) + A2 * Q(2, rho - 1) + A3 * QC(1, (rho + 2) / 2);
      Q(1, my + 1) = A1 * Q(3, my + 1) + A2 * Q(2, my + 1) + A3 * (B1 * QC(1, cmy + 2) + B2 * QC(1, cmy + 1) + B3 * QC(1, cmy));
      Q(1, 2) = A1 * Q(3, 2) + A2 * Q(2, 2) + A3 * (B1 * QC(1, 1) + B2 * QC(1, 2) + B3 * QC(1, 3));
    } else {
      for (int rho = 3; rho <= my + 1; rho += 2) Q(1, rho) = (2.0 / 3.0) * QC(1, (rho + 1) / 2) + (2.0 / 3.0) * Q(2, rho) - (1.0 / 3.0) * Q(2, rho - 1);
      for (int rho = 2; rho <= my; rho += 2) Q(1, rho) = (2.0 / 3.0) * QC(1, (rho + 2) / 2) + (2.0 / 3.0) * Q(2, rho) - (1.0 / 3.0) * Q(2, rho + 1);
    }
  }
  if (fint[1]) {  /* EAST */
    if (qif) {
      for (int rho = 3; rho <= my - 1; rho += 2) Q(mx + 2, rho) = A1 * Q(mx, rho + 2) + A2 * Q(mx + 1, rho + 1) + A3 * QC(cmx + 2, (rho + 1) / 2);
      for (int rho = 4; rho <= my; rho += 2) Q(mx + 2, rho) = A1 * Q(mx, rho - 2) + A2 * Q(mx + 1, rho - 1) + A3 * QC(cmx + 2, (rho + 2) / 2);
      Q(mx + 2, my + 1) = A1 * Q(mx, my + 1) + A2 * Q(mx + 1, my + 1) + A3 * (B1 * QC(cmx + 2, cmy + 2) + B2 * QC(cmx + 2, cmy + 1) + B3 * QC(cmx + 2, cmy));
      Q(mx + 2, 2) = A1 * Q(mx, 2) + A2 * Q(mx + 1, 2) + A3 * (B1 * QC(cmx + 2, 1) + B2 * QC(cmx + 2, 2) + B3 * QC(cmx + 2, 3));
    } else {
      for (int rho = 3; rho <= my + 1; rho += 2) Q(mx + 2, rho) = (2.0 / 3.0) * QC(cmx + 2, (rho + 1) / 2) + (2.0 / 3.0) * Q(mx + 1, rho) - (1.0 / 3.0) * Q(mx + 1, rho - 1);
      for (int rho = 2; rho <= my; rho += 2) Q(mx + 2, rho) = (2.0 / 3.0) * QC(cmx + 2, (rho + 2) / 2) + (2.0 / 3.0) * Q(mx + 1, rho) - (1.0 / 3.0) * Q(mx + 1, rho + 1);
    }
  }
  if (fint[2]) {  /* SOUTH */
    if (qif) {
      for (int kap = 3; kap <= mx - 1; kap += 2) Q(kap, 1) = A1 * Q(kap + 2, 3) + A2 * Q(kap + 1, 2) + A3 * QC((kap + 1) / 2, 1);
      for (int kap = 4; kap <= mx; kap += 2) Q(kap, 1) = A1 * Q(kap - 2, 3) + A2 * Q(kap - 1, 2) + A3 * QC((kap + 2) / 2, 1);
      Q(mx + 1, 1) = A1 * Q(mx + 1, 3) + A2 * Q(mx + 1, 2) + A3 * (B1 * QC(cmx + 2, 1) + B2 * QC(cmx + 1, 1) + B3 * QC(cmx, 1));
      Q(2, 1) = A1 * Q(2, 3) + A2 * Q(2, 2) + A3 * (B1 * QC(1, 1) + B2 * QC(2, 1) + B3 * QC(3, 1));
    } else {
      for (int kap = 3; kap <= mx + 1; kap += 2) Q(kap, 1) = (2.0 / 3.0) * QC((kap + 1) / 2, 1) + (2.0 / 3.0) * Q(kap, 2) - (1.0 / 3.0) * Q(kap - 1, 2);
      for (int kap = 2; kap <= mx; kap += 2) Q(kap, 1) = (2.0 / 3.0) * QC((kap + 2) / 2, 1) + (2.0 / 3.0) * Q(kap, 2) - (1.0 / 3.0) * Q(kap + 1, 2);
    }
  }
  if (fint[3]) {  /* NORTH */
    if (qif) {
      for (int kap = 3; kap <= mx - 1; kap += 2) Q(kap, my + 2) = A1 * Q(kap + 2, my) + A2 * Q(kap + 1, my + 1) + A3 * QC((kap + 1) / 2, cmy + 2);
      for (int kap = 4; kap <= mx; kap += 2) Q(kap, my + 2) = A1 * Q(kap - 2, my) + A2 * Q(kap - 1, my + 1) + A3 * QC((kap + 2) / 2, cmy + 2);
      Q(mx + 1, my + 2) = A1 * Q(mx + 1, my) + A2 * Q(mx + 1, my + 1) + A3 * (B1 * QC(cmx + 2, cmy + 2) + B2 * QC(cmx + 1, cmy + 2) + B3 * QC(cmx, cmy + 2));
      Q(2, my + 2) = A1 * Q(2, my) + A2 * Q(2, my + 1) + A3 * (B1 * QC(1, cmy + 2) + B2 * QC(2, cmy + 2) + B3 * QC(3, cmy + 2));
    } else {
      for (int kap = 3; kap <= mx + 1; kap += 2) Q(kap, my + 2) = (2.0 / 3.0) * QC((kap + 1) / 2, cmy + 2) + (2.0 / 3.0) * Q(kap, my + 1) - (1.0 / 3.0) * Q(kap - 1, my + 1);
      for (int kap = 2; kap <= mx; kap += 2) Q(kap, my + 2) = (2.0 / 3.0) * QC((kap + 2) / 2, cmy + 2) + (2.0 / 3.0) * Q(kap, my + 1) - (1.0 / 3.0) * Q(kap + 1, my + 1);
    }
  }
  /* corners: diagonal stencil */
  if (cCF[0]) Q(1, 1) = qif ? A1 * Q(3, 3) + A2 * Q(2, 2) + A3 * QC(1, 1) : (2.0 / 3.0) * QC(1, 1) + (1.0 / 3.0) * Q(2, 2);
  if (cCF[1]) Q(mx + 2, 1) = qif ? A1 * Q(mx, 3) + A2 * Q(mx + 1, 2) + A3 * QC(cmx + 2, 1) : (2.0 / 3.0) * QC(cmx + 2, 1) + (1.0 / 3.0) * Q(mx + 1, 2);
  if (cCF[2]) Q(1, my + 2) = qif ? A1 * Q(3, my) + A2 * Q(2, my + 1) + A3 * QC(1, cmy + 2) : (2.0 / 3.0) * QC(1, cmy + 2) + (1.0 / 3.0) * Q(2, my + 1);
  if (cCF[3]) Q(mx + 2, my + 2) = qif ? A1 * Q(mx, my) + A2 * Q(mx + 1, my + 1) + A3 * QC(cmx + 2, cmy + 2) : (2.0 / 3.0) * QC(cmx + 2, cmy + 2) + (1.0 / 3.0) * Q(mx + 1, my + 1);
#undef Q
#undef QC
}

/* QC ring <- parent Q (ebTransfer.m:35-55 'ring'; tree: ebtTransfer.m) */
static void ring_patch(OHier *h, const int32_t *r) {
  for (int t = r[PD_RING0]; t < r[PD_RING1]; ++t)
    h->QC[h->ring[2 * t + 1]] = h->Q[h->ring[2 * t]];
}

/* ebFillGhosts (EllipticBSAM/src/ebFillGhosts.m:17-94) */
void oracle_fill_ghosts(OHier *h, int k) {
  const int32_t *L = h->levels + (size_t)(k - 1) * LD;
  const double hx = h->hs[2 * (k - 1)], hy = h->hs[2 * (k - 1) + 1];
  /* 1. coarse-fine interpolation */
  if (k > 1) {
#pragma omp parallel for schedule(dynamic)
    for (int p = L[LD_P0]; p < L[LD_P1]; ++p) {
      const int32_t *r = PR(p);
      int any = 0;
      for (int s = 0; s < 4; ++s) any |= (r[PD_FIW + s] != 0) | (r[PD_CCSW + s] == 3);
      if (!any) continue;
      ring_patch(h, r);
      interp_cf(h, r);
    }
  }
  /* 2. same-level exchange */
#pragma omp parallel for schedule(dynamic)
  for (int p = L[LD_P0]; p < L[LD_P1]; ++p) {
    const int32_t *r = PR(p);
    for (int t = r[PD_SAME0]; t < r[PD_SAME1]; ++t) h->Q[h->same[2 * t + 1]] = h->Q[h->same[2 * t]];
  }
  /* 3. physical boundaries */
#pragma omp parallel for schedule(dynamic)
  for (int p = L[LD_P0]; p < L[LD_P1]; ++p) {
    const int32_t *r = PR(p);
    const int mx = r[PD_MX], my = r[PD_MY];
    const double *g = h->bcg + r[PD_BCGOFF];
    const double *gW = g, *gE = g + my, *gS = g + 2 * my, *gN = g + 2 * my + mx;
#define Q(i, j) QP(r, i, j)
    if (r[PD_BCW] == 1) for (int j = 2; j <= my + 1; ++j) Q(1, j) = (8.0 / 3.0) * gW[j - 2] - 2 * Q(2, j) + (1.0 / 3.0) * Q(3, j);
    else if (r[PD_BCW] == 2) for (int j = 2; j <= my + 1; ++j) Q(1, j) = Q(2, j) + hx * gW[j - 2];
    if (r[PD_BCE] == 1) for (int j = 2; j <= my + 1; ++j) Q(mx + 2, j) = (8.0 / 3.0) * gE[j - 2] - 2 * Q(mx + 1, j) + (1.0 / 3.0) * Q(mx, j);
    else if (r[PD_BCE] == 2) for (int j = 2; j <= my + 1; ++j) Q(mx + 2, j) = Q(mx + 1, j) + hx * gE[j - 2];
    if (r[PD_BCS] == 1) for (int i = 2; i <= mx + 1; ++i) Q(i, 1) = (8.0 / 3.0) * gS[i - 2] - 2 * Q(i, 2) + (1.0 / 3.0) * Q(i, 3);
    else if (r[PD_BCS] == 2) for (int i = 2; i <= mx + 1; ++i) Q(i, 1) = Q(i, 2) + hy * gS[i - 2];
    if (r[PD_BCN] == 1) for (int i = 2; i <= mx + 1; ++i) Q(i, my + 2) = (8.0 / 3.0) * gN[i - 2] - 2 * Q(i, my + 1) + (1.0 / 3.0) * Q(i, my);
    else if (r[PD_BCN] == 2) for (int i = 2; i <= mx + 1; ++i) Q(i, my + 2) = Q(i, my + 1) + hy * gN[i - 2];
    if (r[PD_CCSW] == 1) Q(1, 1) = Q(2, 1) + Q(1, 2) - Q(2, 2);
    if (r[PD_CCSE] == 1) Q(mx + 2, 1) = Q(mx + 1, 1) + Q(mx + 2, 2) - Q(mx + 1, 2);
    if (r[PD_CCNW] == 1) Q(1, my + 2) = Q(2, my + 2) + Q(1, my + 1) - Q(2, my + 1);
    if (r[PD_CCNE] == 1) Q(mx + 2, my + 2) = Q(mx + 1, my + 2) + Q(mx + 2, my + 1) - Q(mx + 1, my + 1);
#undef Q
  }
}

/* relax2d (EllipticBSAM/src/ebKernels.m:37-95), one colour of one patch */
static void relax_patch(OHier *h, const int32_t *r, int color, double hx, double hy) {
  const int mx = r[PD_MX], my = r[PD_MY], par0 = r[PD_PAR0];
  const double *g = h->bcg + r[PD_BCGOFF];
  const double *gW = g, *gE = g + my, *gS = g + 2 * my, *gN = g + 2 * my + mx;
  const double *Fp = h->F + r[PD_COFF], *IDp = h->ID + r[PD_COFF];
  const double *DeW = h->DeW + r[PD_DEWOFF], *DnS = h->DnS + r[PD_DNSOFF];
  const double omega = h->omega;
#define Q(i, j) QP(r, i, j)
  /* partial physical ghosts */
  if (r[PD_BCW] == 1) for (int j = 2; j <= my + 1; ++j) Q(1, j) = (8.0 / 3.0) * gW[j - 2] + (1.0 / 3.0) * Q(3, j);
  else if (r[PD_BCW] == 2) for (int j = 2; j <= my + 1; ++j) Q(1, j) = hx * gW[j - 2];
  if (r[PD_BCE] == 1) for (int j = 2; j <= my + 1; ++j) Q(mx + 2, j) = (8.0 / 3.0) * gE[j - 2] + (1.0 / 3.0) * Q(mx, j);
  else if (r[PD_BCE] == 2) for (int j = 2; j <= my + 1; ++j) Q(mx + 2, j) = hx * gE[j - 2];
  if (r[PD_BCS] == 1) for (int i = 2; i <= mx + 1; ++i) Q(i, 1) = (8.0 / 3.0) * gS[i - 2] + (1.0 / 3.0) * Q(i, 3);
  else if (r[PD_BCS] == 2) for (int i = 2; i <= mx + 1; ++i) Q(i, 1) = hy * gS[i - 2];
  if (r[PD_BCN] == 1) for (int i = 2; i <= mx + 1; ++i) Q(i, my + 2) = (8.0 / 3.0) * gN[i - 2] + (1.0 / 3.0) * Q(i, my);
  else if (r[PD_BCN] == 2) for (int i = 2; i <= mx + 1; ++i) Q(i, my + 2) = hy * gN[i - 2];
  const double hx2 = hx * hx, hy2 = hy * hy;
  /* Candidates are computed from the pre-pass values of the other colour
     only, so in-place strided writes equal the reference's "all candidates,
     then write one colour". */
  const int m = color - 1;
  for (int lj = 1; lj <= my; ++lj) {
    const int li0 = ((1 + lj + par0) % 2 == m) ? 1 : 2;
    for (int li = li0; li <= mx; li += 2) {
      const size_t c = (size_t)(li - 1) + (size_t)(lj - 1) * mx;
      const double tmp = (Fp[c]
          + Q(li + 2, lj + 1) * DeW[li + (size_t)(lj - 1) * (mx + 1)] / hx2
          + Q(li, lj + 1) * DeW[(li - 1) + (size_t)(lj - 1) * (mx + 1)] / hx2
          + Q(li + 1, lj + 2) * DnS[(li - 1) + (size_t)lj * mx] / hy2
          + Q(li + 1, lj) * DnS[(li - 1) + (size_t)(lj - 1) * mx] / hy2) * IDp[c];
      if (omega == 1.0) Q(li + 1, lj + 1) = tmp;
      else Q(li + 1, lj + 1) = omega * tmp + (1 - omega) * Q(li + 1, lj + 1);
    }
  }
#undef Q
}

/* ebRelaxLevel (EllipticBSAM/src/ebRelaxLevel.m:20-38) */
void oracle_relax_level(OHier *h, int k, int nsweeps) {
  const int32_t *L = h->levels + (size_t)(k - 1) * LD;
  const double hx = h->hs[2 * (k - 1)], hy = h->hs[2 * (k - 1) + 1];
  for (int s = 0; s < nsweeps; ++s)
    for (int color = 1; color <= 2; ++color) {
#pragma omp parallel for schedule(dynamic)
      for (int p = L[LD_P0]; p < L[LD_P1]; ++p) relax_patch(h, PR(p), color, hx, hy);
      oracle_fill_ghosts(h, k);
    }
}

/* restrict2 of the interior of patch p into QC interior and the parent Q
   over the footprint (ebTransfer.m:10-33; ebKernels.m:98-102) */
static void restrict_patch(OHier *h, const int32_t *r, int to_parent) {
  const int mx = r[PD_MX], cmx = mx / 2, cmy = r[PD_MY] / 2;
  const int32_t *fp = h->fp + 2 * (size_t)r[PD_FP0];
#define Q(i, j) QP(r, i, j)
  for (int cj = 1; cj <= cmy; ++cj)
    for (int ci = 1; ci <= cmx; ++ci) {
      const int i = 2 * ci, j = 2 * cj;   /* padded index of the (1,1) child */
      const double R = 0.25 * (Q(i, j) + Q(i + 1, j) + Q(i, j + 1) + Q(i + 1, j + 1));
      QCP(r, ci + 1, cj + 1) = R;
      if (to_parent) h->Q[fp[2 * ((ci - 1) + (size_t)(cj - 1) * cmx)]] = R;
    }
#undef Q
}

void oracle_restrict(OHier *h, int k) {
  const int32_t *L = h->levels + (size_t)(k - 1) * LD;
#pragma omp parallel for schedule(dynamic)
  for (int p = L[LD_P0]; p < L[LD_P1]; ++p) restrict_patch(h, PR(p), 1);
}

void oracle_ring(OHier *h, int k) {
  const int32_t *L = h->levels + (size_t)(k - 1) * LD;
#pragma omp parallel for schedule(dynamic)
  for (int p = L[LD_P0]; p < L[LD_P1]; ++p) ring_patch(h, PR(p));
}

/* prolongBilin (ebKernels.m:105-123) of W - QC added to the interior, or
   of W alone written to the interior (init).  'correct' ebTransfer.m:57-71,
   initial guess ebAddLevel.m:26-31. */
static void prolong_patch(OHier *h, const int32_t *r, double *E, int correct) {
  const int mx = r[PD_MX], my = r[PD_MY], cm = mx / 2, cn = my / 2;
  const int32_t *win = h->win + r[PD_WIN0];
  const size_t nw = (size_t)(cm + 2) * (cn + 2);
  for (size_t t = 0; t < nw; ++t) {
    const double w = h->Q[win[t]];
    E[t] = correct ? w - h->QC[r[PD_QCOFF] + t] : w;
  }
#define EW(i, j) E[((i) - 1) + (size_t)((j) - 1) * (cm + 2)]
#define Q(i, j) QP(r, i, j)
  for (int b = 1; b <= cn; ++b)
    for (int a = 1; a <= cm; ++a) {
      const double C = EW(a + 1, b + 1), Wm = EW(a, b + 1), Wp = EW(a + 2, b + 1);
      const double Sm = EW(a + 1, b), Sp = EW(a + 1, b + 2);
      const double Dmm = EW(a, b), Dpm = EW(a + 2, b), Dmp = EW(a, b + 2), Dpp = EW(a + 2, b + 2);
      const double f11 = (9 * C + 3 * Wm + 3 * Sm + Dmm) / 16;
      const double f21 = (9 * C + 3 * Wp + 3 * Sm + Dpm) / 16;
      const double f12 = (9 * C + 3 * Wm + 3 * Sp + Dmp) / 16;
      const double f22 = (9 * C + 3 * Wp + 3 * Sp + Dpp) / 16;
      const int i = 2 * a, j = 2 * b;  /* padded (2a, 2b) = interior (2a-1, 2b-1) */
      if (correct) {
        Q(i, j) = Q(i, j) + f11; Q(i + 1, j) = Q(i + 1, j) + f21;
        Q(i, j + 1) = Q(i, j + 1) + f12; Q(i + 1, j + 1) = Q(i + 1, j + 1) + f22;
      } else {
        Q(i, j) = f11; Q(i + 1, j) = f21; Q(i, j + 1) = f12; Q(i + 1, j + 1) = f22;
      }
    }
#undef EW
#undef Q
}

void oracle_correct(OHier *h, int k, int correct) {
  const int32_t *L = h->levels + (size_t)(k - 1) * LD;
#pragma omp parallel for schedule(dynamic)
  for (int p = L[LD_P0]; p < L[LD_P1]; ++p) {
    const int32_t *r = PR(p);
    double *E = (double *)malloc(sizeof(double) * (size_t)(r[PD_MX] / 2 + 2) * (r[PD_MY] / 2 + 2));
    prolong_patch(h, r, E, correct);
    free(E);
  }
}

/* op2d (ebKernels.m:13-25) at interior cell (li, lj) of a padded array */
static inline double op_cell(const double *Qa, int ldq, const double *DeW, const double *DnS,
                             const double *CC, int mx, int li, int lj, double hx, double hy) {
  /* Qa is the padded array; (li, lj) are 1-based interior indices */
#define QA(i, j) Qa[((i) - 1) + (size_t)((j) - 1) * ldq]
  const double feE = DeW[li + (size_t)(lj - 1) * (mx + 1)] * (QA(li + 2, lj + 1) - QA(li + 1, lj + 1));
  const double feW = DeW[(li - 1) + (size_t)(lj - 1) * (mx + 1)] * (QA(li + 1, lj + 1) - QA(li, lj + 1));
  const double fnN = DnS[(li - 1) + (size_t)lj * mx] * (QA(li + 1, lj + 2) - QA(li + 1, lj + 1));
  const double fnS = DnS[(li - 1) + (size_t)(lj - 1) * mx] * (QA(li + 1, lj + 1) - QA(li + 1, lj));
  return -(feE - feW) / (hx * hx) - (fnN - fnS) / (hy * hy) + CC[(li - 1) + (size_t)(lj - 1) * mx] * QA(li + 1, lj + 1);
#undef QA
}

/* ebFaceCorrections (EllipticBSAM/src/ebFaceCorrections.m:18-61): the
   correction value of coarse face j (0-based) on face f (0 W,1 E,2 S,3 N) */
static double face_corr(const OHier *h, const int32_t *r, int f, int j, double hcx2, double hcy2) {
  const int mx = r[PD_MX], my = r[PD_MY], cmx = mx / 2, cmy = my / 2;
  const double *DeW = h->DeW + r[PD_DEWOFF], *DnS = h->DnS + r[PD_DNSOFF];
  const double *cfd = h->cfd + r[PD_CFDOFF];
#define Q(i, jj) QP(r, i, jj)
#define QC(i, jj) QCP(r, i, jj)
#define DEW(i, jj) DeW[((i) - 1) + (size_t)((jj) - 1) * (mx + 1)]
#define DNS(i, jj) DnS[((i) - 1) + (size_t)((jj) - 1) * mx]
  const int J = j + 1;  /* 1-based coarse face index */
  switch (f) {
    case 0:
      return (DEW(1, 2 * J - 1) * (Q(2, 2 * J) - Q(1, 2 * J)) + DEW(1, 2 * J) * (Q(2, 2 * J + 1) - Q(1, 2 * J + 1))
              + cfd[j] * (QC(1, J + 1) - QC(2, J + 1))) / hcx2;
    case 1:
      return (DEW(mx + 1, 2 * J - 1) * (Q(mx + 1, 2 * J) - Q(mx + 2, 2 * J)) + DEW(mx + 1, 2 * J) * (Q(mx + 1, 2 * J + 1) - Q(mx + 2, 2 * J + 1))
              + cfd[cmy + j] * (QC(cmx + 2, J + 1) - QC(cmx + 1, J + 1))) / hcx2;
    case 2:
      return (DNS(2 * J - 1, 1) * (Q(2 * J, 2) - Q(2 * J, 1)) + DNS(2 * J, 1) * (Q(2 * J + 1, 2) - Q(2 * J + 1, 1))
              + cfd[2 * cmy + j] * (QC(J + 1, 1) - QC(J + 1, 2))) / hcy2;
    default:
      return (DNS(2 * J - 1, my + 1) * (Q(2 * J, my + 1) - Q(2 * J, my + 2)) + DNS(2 * J, my + 1) * (Q(2 * J + 1, my + 1) - Q(2 * J + 1, my + 2))
              + cfd[2 * cmy + cmx + j] * (QC(J + 1, cmy + 2) - QC(J + 1, cmy + 1))) / hcy2;
  }
#undef Q
#undef QC
#undef DEW
#undef DNS
}

/* ebCoarseLoad (EllipticBSAM/src/ebCoarseLoad.m:17-46) + ebParentCoeffs */
void oracle_coarse_load(OHier *h, int k) {
  const int32_t *L = h->levels + (size_t)(k - 1) * LD;
  const double hx = h->hs[2 * (k - 1)], hy = h->hs[2 * (k - 1) + 1];
  const double hcx = h->hs[2 * (k - 2)], hcy = h->hs[2 * (k - 2) + 1];
#pragma omp parallel for schedule(dynamic)
  for (int p = L[LD_P0]; p < L[LD_P1]; ++p) {
    const int32_t *r = PR(p);
    const int mx = r[PD_MX], my = r[PD_MY], cmx = mx / 2, cmy = my / 2;
    const double *Qp = h->Q + r[PD_QOFF], *Fp = h->F + r[PD_COFF];
    const double *DeW = h->DeW + r[PD_DEWOFF], *DnS = h->DnS + r[PD_DNSOFF], *CC = h->CC + r[PD_COFF];
    const double *PDeW = h->pcoef + r[PD_PCOFF];
    const double *PDnS = PDeW + (size_t)(cmx + 1) * cmy;
    const double *PCC = PDnS + (size_t)cmx * (cmy + 1);
    const double *QCp = h->QC + r[PD_QCOFF];
    const int32_t *fp = h->fp + 2 * (size_t)r[PD_FP0];
    for (int cj = 1; cj <= cmy; ++cj)
      for (int ci = 1; ci <= cmx; ++ci) {
        double RF[4];
        int t = 0;
        for (int dj = 0; dj < 2; ++dj)
          for (int di = 0; di < 2; ++di) {
            const int li = 2 * ci - 1 + di, lj = 2 * cj - 1 + dj;
            RF[t++] = Fp[(li - 1) + (size_t)(lj - 1) * mx] - op_cell(Qp, mx + 2, DeW, DnS, CC, mx, li, lj, hx, hy);
          }
        /* restrict2 order: (1,1) + (2,1) + (1,2) + (2,2) */
        const double rr = 0.25 * (RF[0] + RF[1] + RF[2] + RF[3]);
        const double lc = op_cell(QCp, cmx + 2, PDeW, PDnS, PCC, cmx, ci, cj, hcx, hcy);
        h->F[fp[2 * ((ci - 1) + (size_t)(cj - 1) * cmx) + 1]] = rr + lc;
      }
  }
  if (!h->mass_corr) return;
  const double hcx2 = hcx * hcx, hcy2 = hcy * hcy;
  /* ordered scatter-add: patch p ascending, faces W, E, S, N */
  for (int p = L[LD_P0]; p < L[LD_P1]; ++p) {
    const int32_t *r = PR(p);
    const int cmx = r[PD_MX] / 2, cmy = r[PD_MY] / 2;
    const int32_t *corr = h->corr + r[PD_CORR0];
    int o = 0;
    for (int f = 0; f < 4; ++f) {
      const int nn = (f < 2) ? cmy : cmx;
      for (int j = 0; j < nn; ++j) {
        const int tgt = corr[o + j];
        if (tgt >= 0) h->F[tgt] = h->F[tgt] + face_corr(h, r, f, j, hcx2, hcy2);
      }
      o += nn;
    }
  }
}

/* ebCoarsest('solve') (EllipticBSAM/src/ebCoarsest.m:79-91): u = Ainv*rhs
   in the fixed order shared with the device kernel */
void oracle_coarsest(OHier *h) {
  const int32_t *r = PR(0);
  const int n1 = r[PD_MX], n2 = r[PD_MY], N = n1 * n2;
  double *rhs = (double *)malloc(sizeof(double) * N);
  for (int i = 0; i < N; ++i) rhs[i] = h->F[r[PD_COFF] + i] + h->bcRhs[i];
#pragma omp parallel for schedule(static)
  for (int row = 0; row < N; ++row) {
    double acc[32];
    const double *a = h->Ainv + (size_t)row * N;
    for (int l = 0; l < 32; ++l) {
      double s = 0.0;
      for (int c = l; c < N; c += 32) s = s + a[c] * rhs[c];
      acc[l] = s;
    }
    for (int off = 16; off >= 1; off >>= 1)
      for (int l = 0; l < off; ++l) acc[l] = acc[l] + acc[l + off];
    const int i = row % n1 + 1, j = row / n1 + 1;
    QP(r, i + 1, j + 1) = acc[0];
  }
  free(rhs);
  oracle_fill_ghosts(h, 1);
}

/* ebVcycle (EllipticBSAM/src/ebVcycle.m:16-35) */
void oracle_vcycle(OHier *h, int k) {
  if (k == 1) { oracle_coarsest(h); return; }
  oracle_relax_level(h, k, h->npre);
  oracle_restrict(h, k);
  oracle_fill_ghosts(h, k - 1);
  oracle_ring(h, k);
  oracle_coarse_load(h, k);
  oracle_vcycle(h, k - 1);
  oracle_correct(h, k, 1);
  oracle_fill_ghosts(h, k);
  oracle_relax_level(h, k, h->npost);
}

/* ebTransfer(H,0,'filldown') (ebTransfer.m:73-79) */
void oracle_filldown(OHier *h) {
  for (int kk = h->nlev; kk >= 2; --kk) {
    oracle_restrict(h, kk);
    oracle_fill_ghosts(h, kk - 1);
  }
}

/* ebCompResidual (EllipticBSAM/src/ebCompResidual.m:15-85) */
void oracle_comp_residual(OHier *h, ORes *res) {
  const int r0 = h->root_idx;
  size_t ncells = (size_t)h->levels[(size_t)(h->nlev - 1) * LD + LD_CELL1];
  if (h->mass_corr) {
    for (int k = (r0 + 1 > 2 ? r0 + 1 : 2); k <= h->nlev; ++k) {
      const int32_t *L = h->levels + (size_t)(k - 1) * LD;
      oracle_ring(h, k);
#pragma omp parallel for schedule(dynamic)
      for (int p = L[LD_P0]; p < L[LD_P1]; ++p) restrict_patch(h, PR(p), 0);
    }
  }
  /* r = FTrue - op(Q); then r(dst) += vals, chunk by chunk: the chunks of a
     target are its corrections in order (k, p ascending, face W,E,S,N), and
     each add rounds, so they are replayed in that order onto r. */
  double linf = 0, l2sq = 0, fnorm = 0;
  long long ncell = 0;
  /* collect correction values per target in order */
  int *cnt = NULL, *start = NULL, *fill = NULL;
  double *vals = NULL;
  if (h->mass_corr) {
    cnt = (int *)calloc(ncells + 1, sizeof(int));
    for (int k = r0 + 1; k <= h->nlev; ++k) {
      const int32_t *L = h->levels + (size_t)(k - 1) * LD;
      for (int p = L[LD_P0]; p < L[LD_P1]; ++p) {
        const int32_t *r = PR(p);
        const int n = r[PD_MX] + r[PD_MY];
        for (int t = 0; t < n; ++t) if (h->corr[r[PD_CORR0] + t] >= 0) cnt[h->corr[r[PD_CORR0] + t]]++;
      }
    }
    start = (int *)malloc(sizeof(int) * (ncells + 1));
    start[0] = 0;
    for (size_t c = 0; c < ncells; ++c) start[c + 1] = start[c] + cnt[c];
    fill = (int *)calloc(ncells, sizeof(int));
    vals = (double *)malloc(sizeof(double) * (start[ncells] + 1));
    for (int k = r0 + 1; k <= h->nlev; ++k) {
      const int32_t *L = h->levels + (size_t)(k - 1) * LD;
      const double hcx = h->hs[2 * (k - 2)], hcy = h->hs[2 * (k - 2) + 1];
      for (int p = L[LD_P0]; p < L[LD_P1]; ++p) {
        const int32_t *r = PR(p);
        const int cmx = r[PD_MX] / 2, cmy = r[PD_MY] / 2;
        int o = 0;
        for (int f = 0; f < 4; ++f) {
          const int nn = (f < 2) ? cmy : cmx;
          for (int j = 0; j < nn; ++j) {
            const int tgt = h->corr[r[PD_CORR0] + o + j];
            if (tgt >= 0) vals[start[tgt] + fill[tgt]++] = face_corr(h, r, f, j, hcx * hcx, hcy * hcy);
          }
          o += nn;
        }
      }
    }
  }
  for (int k = r0; k <= h->nlev; ++k) {
    const int32_t *L = h->levels + (size_t)(k - 1) * LD;
    const double hx = h->hs[2 * (k - 1)], hy = h->hs[2 * (k - 1) + 1];
    const double area = hx * hy;
    const int np = L[LD_P1] - L[LD_P0];
    double *pl = (double *)calloc((size_t)np * 3, sizeof(double));
    long long *pn = (long long *)calloc((size_t)np, sizeof(long long));
#pragma omp parallel for schedule(dynamic)
    for (int pi = 0; pi < np; ++pi) {
      const int32_t *r = PR(L[LD_P0] + pi);
      const int mx = r[PD_MX], my = r[PD_MY];
      const double *Qp = h->Q + r[PD_QOFF];
      const size_t co = r[PD_COFF];
      double li = 0, sq = 0, fn = 0;
      long long nc = 0;
      for (int lj = 1; lj <= my; ++lj)
        for (int lii = 1; lii <= mx; ++lii) {
          const size_t c = co + (lii - 1) + (size_t)(lj - 1) * mx;
          double rr = h->FTrue[c] - op_cell(Qp, mx + 2, h->DeW + r[PD_DEWOFF], h->DnS + r[PD_DNSOFF], h->CC + co, mx, lii, lj, hx, hy);
          if (cnt) for (int t = start[c]; t < start[c + 1]; ++t) rr = rr + vals[t];
          if (h->covered[c]) continue;
          const double a = fabs(rr);
          if (a > li) li = a;
          sq = sq + rr * rr;
          const double fa = fabs(h->FTrue[c]);
          if (fa > fn) fn = fa;
          ++nc;
        }
      pl[3 * pi] = li; pl[3 * pi + 1] = sq; pl[3 * pi + 2] = fn; pn[pi] = nc;
    }
    for (int pi = 0; pi < np; ++pi) {
      if (pn[pi] == 0) continue;
      if (pl[3 * pi] > linf) linf = pl[3 * pi];
      l2sq = l2sq + pl[3 * pi + 1] * area;
      if (pl[3 * pi + 2] > fnorm) fnorm = pl[3 * pi + 2];
      ncell += pn[pi];
    }
    free(pl); free(pn);
  }
  free(cnt); free(start); free(fill); free(vals);
  res->linf = linf;
  res->l2 = sqrt(l2sq);
  res->fnorm = fnorm > DBL_MIN ? fnorm : DBL_MIN;
  res->rel = linf / res->fnorm;
  res->ncell = ncell;
}

/* ebSolveCycles (EllipticBSAM/src/ebSolveCycles.m:8-70).  Returns the number
   of V-cycles; resHist receives vcycles+1 entries (capacity hist_cap). */
int oracle_solve_cycles(OHier *h, double *resHist, int hist_cap, double *finalRel, long long *visibleCells) {
  for (int k = 1; k <= h->nlev; ++k) oracle_fill_ghosts(h, k);
  ORes res;
  oracle_comp_residual(h, &res);
  int nh = 0;
  if (nh < hist_cap) resHist[nh] = res.linf;
  ++nh;
  double rel = res.rel;
  int it = 0;
  const size_t ncells = (size_t)h->levels[(size_t)(h->nlev - 1) * LD + LD_CELL1];
  while (it < h->max_vcycles && rel > h->rel_tol) {
    ++it;
    memcpy(h->F, h->FTrue, sizeof(double) * ncells);
    oracle_vcycle(h, h->nlev);
    oracle_filldown(h);
    oracle_comp_residual(h, &res);
    if (nh < hist_cap) resHist[nh] = res.linf;
    ++nh;
    rel = res.rel;
  }
  *finalRel = rel;
  *visibleCells = res.ncell;
  return it;
}

/* ebCompositeMean (EllipticBSAM/src/ebCompositeMean.m:4-23), solution field */
void oracle_composite_mean(OHier *h, double *mean, double *area_out) {
  double tot = 0, area = 0;
  for (int k = h->root_idx; k <= h->nlev; ++k) {
    const int32_t *L = h->levels + (size_t)(k - 1) * LD;
    const double da = h->hs[2 * (k - 1)] * h->hs[2 * (k - 1) + 1];
    for (int p = L[LD_P0]; p < L[LD_P1]; ++p) {
      const int32_t *r = PR(p);
      const int mx = r[PD_MX], my = r[PD_MY];
      double s = 0;
      long long nv = 0;
      for (int j = 1; j <= my; ++j)
        for (int i = 1; i <= mx; ++i) {
          const size_t c = r[PD_COFF] + (i - 1) + (size_t)(j - 1) * mx;
          if (h->covered[c]) continue;
          s = s + QP(r, i + 1, j + 1);
          ++nv;
        }
      tot = tot + s * da;
      area = area + (double)nv * da;
    }
  }
  *mean = tot / (area > DBL_MIN ? area : DBL_MIN);
  *area_out = area;
}

/* ebMassCheck (EllipticBSAM/src/ebMassCheck.m:15-66) */
void oracle_mass_check(OHier *h, double out[4]) {
  double lhs = 0, scale = 0, rhs = 0;
  for (int k = h->root_idx; k <= h->nlev; ++k) {
    const int32_t *L = h->levels + (size_t)(k - 1) * LD;
    const double hx = h->hs[2 * (k - 1)], hy = h->hs[2 * (k - 1) + 1], da = hx * hy;
    for (int p = L[LD_P0]; p < L[LD_P1]; ++p) {
      const int32_t *r = PR(p);
      const int mx = r[PD_MX], my = r[PD_MY];
      const size_t co = r[PD_COFF];
      const double *DeW = h->DeW + r[PD_DEWOFF], *DnS = h->DnS + r[PD_DNSOFF];
      double s = 0, sa = 0;
      for (int j = 1; j <= my; ++j)
        for (int i = 1; i <= mx; ++i) {
          const size_t c = co + (i - 1) + (size_t)(j - 1) * mx;
          if (h->covered[c]) continue;
          s = s + (h->CC[c] * QP(r, i + 1, j + 1) - h->FTrue[c]);
          sa = sa + fabs(h->FTrue[c]);
        }
      lhs = lhs + s * da;
      scale = scale + sa * da;
#define COV(i, j) h->covered[co + ((i) - 1) + (size_t)((j) - 1) * mx]
      if (r[PD_BCW] > 0) { double f = 0; for (int j = 1; j <= my; ++j) if (!COV(1, j)) f = f + DeW[(size_t)(j - 1) * (mx + 1)] * (QP(r, 1, j + 1) - QP(r, 2, j + 1)) / hx; rhs = rhs + f * hy; }
      if (r[PD_BCE] > 0) { double f = 0; for (int j = 1; j <= my; ++j) if (!COV(mx, j)) f = f + DeW[mx + (size_t)(j - 1) * (mx + 1)] * (QP(r, mx + 2, j + 1) - QP(r, mx + 1, j + 1)) / hx; rhs = rhs + f * hy; }
      if (r[PD_BCS] > 0) { double f = 0; for (int i = 1; i <= mx; ++i) if (!COV(i, 1)) f = f + DnS[i - 1] * (QP(r, i + 1, 1) - QP(r, i + 1, 2)) / hy; rhs = rhs + f * hx; }
      if (r[PD_BCN] > 0) { double f = 0; for (int i = 1; i <= mx; ++i) if (!COV(i, my)) f = f + DnS[(i - 1) + (size_t)my * mx] * (QP(r, i + 1, my + 2) - QP(r, i + 1, my + 1)) / hy; rhs = rhs + f * hx; }
#undef COV
    }
  }
  out[0] = lhs; out[1] = rhs; out[2] = lhs - rhs;
  double m = scale;
  if (fabs(lhs) > m) m = fabs(lhs);
  if (fabs(rhs) > m) m = fabs(rhs);
  if (DBL_MIN > m) m = DBL_MIN;
  out[3] = fabs(lhs - rhs) / m;
}

/* ---------------------------------------------------------------------- */
/* construction: the arrays stay owned by the caller                         */
OHier *oracle_new(int nlev, int root_idx, int npatch, const int32_t *levels, const double *hs,
                  const int32_t *patches, double *Q, double *F, double *FTrue, double *QC,
                  const double *CC, const double *ID, const double *DeW, const double *DnS,
                  const double *bcg, const double *cfd, const double *pcoef, const uint8_t *covered,
                  const int32_t *same, const int32_t *ring, const int32_t *win, const int32_t *fp,
                  const int32_t *corr, const double *Ainv, const double *bcRhs, int ncoarse,
                  int npre, int npost, double omega, int qif, int mass_corr, int max_vcycles,
                  double rel_tol) {
  OHier *h = (OHier *)calloc(1, sizeof(OHier));
  h->nlev = nlev; h->root_idx = root_idx; h->npatch = npatch;
  h->levels = levels; h->hs = hs; h->patches = patches;
  h->Q = Q; h->F = F; h->FTrue = FTrue; h->QC = QC;
  h->CC = CC; h->ID = ID; h->DeW = DeW; h->DnS = DnS; h->bcg = bcg; h->cfd = cfd; h->pcoef = pcoef;
  h->covered = covered; h->same = same; h->ring = ring; h->win = win; h->fp = fp; h->corr = corr;
  h->Ainv = Ainv; h->bcRhs = bcRhs; h->ncoarse = ncoarse;
  h->npre = npre; h->npost = npost; h->omega = omega; h->qif = qif; h->mass_corr = mass_corr;
  h->max_vcycles = max_vcycles; h->rel_tol = rel_tol;
  return h;
}

void oracle_free(OHier *h) { free(h); }

void oracle_residual(OHier *h, double out[5]) {
  ORes r;
  oracle_comp_residual(h, &r);
  out[0] = r.linf; out[1] = r.l2; out[2] = r.fnorm; out[3] = r.rel; out[4] = (double)r.ncell;
}
