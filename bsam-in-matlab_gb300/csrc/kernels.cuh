// kernels.cuh -- sm_103a kernels of the BSAM adaptive FAS V-cycle (FP64).
//
// Every kernel restates one step of the reference's MATLAB solve path in the
// reference's floating-point operation order (the library is compiled with
// --fmad=false, so no multiply-add is contracted).  Work is flattened per
// level over all patches: a level's items (colour cells, cells, coarse
// cells, ...) are numbered consecutively patch after patch and cut into
// 256-item blocks; `blk_p0[b]` names the patch that holds block b's first
// item, `beg[p]..beg[p+1]` the items of patch p.
//
// Memory layout in HBM: one array per field with every patch of every level
// concatenated, each patch column-major (x fastest) like the reference; the
// solution Q and the coarse shadows QC carry their one-cell ghost frame.
//
// Launch chaining (programmatic dependent launch): every kernel opens with
// griddepcontrol.launch_dependents, so the next kernel of the V-cycle is
// scheduled while this one drains, then loads what no kernel of the solve
// writes (patch records, coefficients, ghost rules, index tables) and only
// then executes griddepcontrol.wait, after which it reads and writes the
// solution state.  Every thread executes the wait before it exits, so no
// kernel completes before its predecessor.
#pragma once
#include <cooperative_groups.h>
#include <cstdint>
#include <cuda_runtime.h>

#include "stencil.cuh"

namespace bsam {

__device__ __forceinline__ void chain_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void chain_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void chain_in() {
  chain_trigger();
  chain_wait();
}

// a solution load; kCG: from L2 (ld.global.cg), for kernels whose blocks
// read values other blocks of the same launch wrote after a cluster barrier
// (another SM's L1 may hold an older copy of the line)
template <bool kCG, class T>
__device__ __forceinline__ T ld_sol(const T *p) {
  if constexpr (kCG) return __ldcg(p);
  else return *p;
}

// per-patch metadata on the device
struct PatchD {
  int mx, my, par0, level;
  int q_off, c_off, dew_off, dns_off;
  int qc_off, bcg_off, cfd_off, pc_off;
  int win_off, fp_off, corr_off, pe_off;   // pe_off: perimeter ghost-rule table
  int bc[4];
  int inst;                    // instance of a batch (0 for a single hierarchy)
  int pflags;                  // bit0: level >= the instance's root (in the norms)
                               // bit1: QC refreshed by the residual (level >= root+1)
  int ilo, jlo;                // 1-based origin of the patch box in the level's index space
};

// the arrays one V-cycle works on, in its value type T: the FP64 solve
// (T = double) or the FP32 correction cycle of the mixed form (T = float:
// Q is the correction, F its right-hand side, coefficients FP32 copies)
template <class T>
struct FieldsT {
  T *Q, *F, *QC;
  const double *FTrue;         // FP64 source (residual only)
  const T *CC, *ID, *DeW, *DnS, *bcg, *cfd, *pcoef;
  const uint8_t *flags;        // bit0 covered by a finer level, bit1 correction target
  const int *win, *fp;         // window gathers, footprint scatters (2 ints/cell)
  const int *active;           // per instance: 1 while its V-cycles continue (below)
};
// `active` is written only by k_residual_final, the last kernel of a launch
// chain, and the host synchronises before the next chain (or writes it with
// a stream-ordered copy).  Within a chain no kernel can still be in its
// pre-wait part when k_residual_final's body runs (every kernel completes
// only after its predecessor), so kernels read `active` before
// griddepcontrol.wait and the blocks of a frozen instance skip their loads.
using Fields = FieldsT<double>;

// FP64 view of a value of either type (a no-op for double)
template <class T>
__device__ __forceinline__ double dbl(T x) { return (double)x; }

// one level's work decomposition for one kind of item
struct Decomp {
  const int *beg;              // [np+1] item prefix per patch (level-local)
  const int *blk_p0;           // [nblocks] first patch of each block
  int n, nblocks;
};

struct LevelD {
  const PatchD *patches;       // this level's patches
  double hx, hy, hx2, hy2, ihx2, ihy2;   // ihx2 = 1/hx2 (used only when exact)
  int pow2;                    // hx2 and hy2 are powers of two
  float fhx, fhy, fhx2, fhy2;  // FP32 copies for the correction cycle
};

// the level's cell sizes in the cycle's value type
template <class T> struct LevelH {
  T hx, hy, hx2, hy2;
};
__device__ __forceinline__ LevelH<double> level_h(const LevelD &L, double) { return {L.hx, L.hy, L.hx2, L.hy2}; }
__device__ __forceinline__ LevelH<float> level_h(const LevelD &L, float) { return {L.fhx, L.fhy, L.fhx2, L.fhy2}; }

// `b` is the block index within the decomposition
__device__ __forceinline__ int find_patch(const Decomp &D, int b, int g) {
  int p = __ldg(D.blk_p0 + b);
  while (g >= __ldg(D.beg + p + 1)) ++p;
  return p;
}

__device__ __forceinline__ double divr(double x, double h2, double ih2, int pow2) {
  return pow2 ? x * ih2 : x / h2;
}

__device__ __forceinline__ double op_cell_r(const double *__restrict__ Qa, int ldq, const double *__restrict__ DeW,
                                            const double *__restrict__ DnS, double cc, int mx, int li, int lj,
                                            const LevelD &L) {
  return L.pow2 ? op_cell<true>(Qa, ldq, DeW, DnS, cc, mx, li, lj, L.hx2, L.hy2, L.ihx2, L.ihy2)
                : op_cell<false>(Qa, ldq, DeW, DnS, cc, mx, li, lj, L.hx2, L.hy2, L.ihx2, L.ihy2);
}

// ---------------------------------------------------------------------------
// Ghost rules (EllipticBSAM/src/ebFillGhosts.m:17-94, ebInterpCf.m:36-154).
// The three ordered stages (coarse-fine interpolation, same-level copy,
// physical closure) are resolved on the host into one final rule per ghost
// cell.  Value rules read only interior cells, parent cells (the coarse
// window is read from the parent's Q, which is what the QC ring holds) or
// boundary data; a physical corner evaluates its two face-ghost rules
// itself, so a level's ghost frame is filled in one pass.
enum GhostType : int8_t {
  G_COPY = 0, G_QIF = 1, G_QIF_END = 2, G_LIF = 3, G_LIF_CORNER = 4,
  G_DIRICHLET = 5, G_NEUMANN = 6, G_RING = 7, G_PHYS_CORNER = 8
};

struct GhostItems {
  const int8_t *type;
  const int *dst, *a, *b, *c, *d, *e;
  const int *inst;             // instance per item (batches only, else null)
};

// the value of a COPY / QIF / QIF_END / LIF rule from its five operands
template <class T>
__device__ __forceinline__ T rule_value(int type, T qa, T qb, T qc, T qd, T qe) {
  const T A1 = T(-1.0 / 5.0), A2 = T(2.0 / 3.0), A3 = T(8.0 / 15.0);
  const T B1 = T(5.0 / 32.0), B2 = T(15.0 / 16.0), B3 = T(-3.0 / 32.0);
  const T c23 = T(2.0 / 3.0), c13 = T(1.0 / 3.0);
  switch (type) {
    case G_COPY: return qa;
    case G_QIF: return (A1 * qa + A2 * qb) + A3 * qc;
    case G_QIF_END: return (A1 * qa + A2 * qb) + A3 * ((B1 * qc + B2 * qd) + B3 * qe);
    default: return (c23 * qc + c23 * qa) - c13 * qb;   // G_LIF
  }
}

template <class T, bool kCG = false>
__device__ __forceinline__ T eval_rule(const GhostItems &G, int i, const T *Q, const T *bcg, T hx, T hy) {
  const T A1 = T(-1.0 / 5.0), A2 = T(2.0 / 3.0), A3 = T(8.0 / 15.0);
  const T B1 = T(5.0 / 32.0), B2 = T(15.0 / 16.0), B3 = T(-3.0 / 32.0);
  const T c23 = T(2.0 / 3.0), c13 = T(1.0 / 3.0), c83 = T(8.0 / 3.0);
  const int a = G.a[i];
  auto q = [&](int j) { return ld_sol<kCG>(Q + j); };
  switch (G.type[i]) {
    case G_COPY: return q(a);
    case G_QIF: return (A1 * q(a) + A2 * q(G.b[i])) + A3 * q(G.c[i]);
    case G_QIF_END:
      return (A1 * q(a) + A2 * q(G.b[i])) + A3 * ((B1 * q(G.c[i]) + B2 * q(G.d[i])) + B3 * q(G.e[i]));
    case G_LIF: return (c23 * q(G.c[i]) + c23 * q(a)) - c13 * q(G.b[i]);
    case G_LIF_CORNER: return c23 * q(G.c[i]) + c13 * q(a);
    case G_DIRICHLET: return (c83 * bcg[G.e[i]] - 2 * q(a)) + c13 * q(G.b[i]);
    default: return q(a) + (G.b[i] ? hy : hx) * bcg[G.e[i]];   // G_NEUMANN
  }
}

// one ghost item: its final value (or the QC ring refresh)
template <class T, bool kCG = false>
__device__ __forceinline__ void ghost_item(const GhostItems &G, int i, int8_t ty, int dst, T *Q, T *QC, const T *bcg,
                                           T hx, T hy) {
  if (ty == G_RING) {
    QC[dst] = ld_sol<kCG>(Q + G.a[i]);
  } else if (ty == G_PHYS_CORNER) {
    // (face ghost 1 + face ghost 2) - interior, the face ghosts evaluated by
    // their own final rules (ebFillGhosts.m:84-89 reads them after stage 3)
    const T v1 = eval_rule<T, kCG>(G, G.a[i], Q, bcg, hx, hy);
    const T v2 = eval_rule<T, kCG>(G, G.b[i], Q, bcg, hx, hy);
    Q[dst] = (v1 + v2) - ld_sol<kCG>(Q + G.c[i]);
  } else {
    Q[dst] = eval_rule<T, kCG>(G, i, Q, bcg, hx, hy);
  }
}

// A ghost item in two stages, so that every load it needs is in flight at
// once: ghost_prep reads the item's static indices (before a kernel's
// programmatic-launch wait), ghost_apply requests all of its solution
// operands and its boundary value before it looks at the rule's kind, so
// the lanes of a warp that fill different kinds of ghosts wait for one round
// of loads together.  Operand slots a kind does not read repeat its first
// operand.  A physical corner evaluates its two face rules as ghost_item does.
//
// GhostAlt: the operands of a level's ghost items for the fill that follows
// the restriction of the level above into it, fused into one launch with
// that restriction (k_restrict_fill).  A solution operand that the
// restriction overwrites (a cell under the finer level's footprint) is coded
// -1 - j, and the item forms its value itself from the four fine cells of
// entry j of `rt` with restrict_cell's arithmetic -- the value the
// restriction stores -- so the fill reads nothing the same launch writes.
struct GhostAlt {
  const int *a, *b, *c;        // operand slots (d and e are parent cells: never restricted)
  const int2 *rt;              // (first fine cell in Q, fine row stride)
};

struct GhostPrep {
  int8_t ty;
  int dst, a, b, c, d, e, g, nb;   // g: boundary-data index (-1: none); nb: Neumann side flag
};

template <bool kAlt = false>
__device__ __forceinline__ GhostPrep ghost_prep(const GhostItems &G, int i, int8_t ty, int dst,
                                                const GhostAlt *A = nullptr) {
  GhostPrep P;
  P.ty = ty;
  P.dst = dst;
  const int a = kAlt ? __ldg(A->a + i) : __ldg(G.a + i);
  P.a = a;
  const bool ub = ty == G_QIF || ty == G_QIF_END || ty == G_LIF || ty == G_DIRICHLET;
  const bool uc = ty == G_QIF || ty == G_QIF_END || ty == G_LIF || ty == G_LIF_CORNER;
  const bool ue = ty == G_QIF_END;
  P.b = ub ? (kAlt ? __ldg(A->b + i) : __ldg(G.b + i)) : a;
  P.c = uc ? (kAlt ? __ldg(A->c + i) : __ldg(G.c + i)) : a;
  // d and e (parent cells of QIF_END) are read directly: unused, they
  // repeat the item's plain first operand (a cell of Q in every kind that
  // reaches ghost_value)
  const int pa = kAlt ? __ldg(G.a + i) : a;
  P.d = ue ? __ldg(G.d + i) : pa;
  P.e = ue ? __ldg(G.e + i) : pa;
  P.g = (ty == G_DIRICHLET || ty == G_NEUMANN) ? __ldg(G.e + i) : -1;
  P.nb = ty == G_NEUMANN ? __ldg(G.b + i) : 0;
  return P;
}

// a solution operand: a cell of Q, or (code < 0, fused fills only) the
// restriction of its four fine cells
template <class T, bool kCG, bool kAlt>
__device__ __forceinline__ T ghost_operand(const T *Q, int code, const GhostAlt *A) {
  if (kAlt && code < 0) {
    const int2 r = __ldg(A->rt + (-1 - code));
    const T *q = Q + r.x;
    return T(0.25) * (((ld_sol<kCG>(q) + ld_sol<kCG>(q + 1)) + ld_sol<kCG>(q + r.y)) + ld_sol<kCG>(q + r.y + 1));
  }
  return ld_sol<kCG>(Q + code);
}

// a ghost's value from its operands and boundary datum (eval_rule's
// arithmetic, every kind but the ring refresh and the physical corner)
template <class T>
__device__ __forceinline__ T ghost_formula(int ty, T qa, T qb, T qc, T qd, T qe, T g, int nb, T hx, T hy) {
  const T c23 = T(2.0 / 3.0), c13 = T(1.0 / 3.0), c83 = T(8.0 / 3.0);
  switch (ty) {
    case G_LIF_CORNER: return c23 * qc + c13 * qa;
    case G_DIRICHLET: return (c83 * g - 2 * qa) + c13 * qb;
    case G_NEUMANN: return qa + (nb ? hy : hx) * g;
    default: return rule_value<T>(ty, qa, qb, qc, qd, qe);   // COPY, QIF, QIF_END, LIF
  }
}

// the value of a prepared item that is not a ring refresh or a corner
template <class T, bool kCG, bool kAlt>
__device__ __forceinline__ T ghost_value(const GhostPrep &P, const T *Q, const T *bcg, T hx, T hy,
                                         const GhostAlt *A) {
  const T qa = ghost_operand<T, kCG, kAlt>(Q, P.a, A), qb = ghost_operand<T, kCG, kAlt>(Q, P.b, A);
  const T qc = ghost_operand<T, kCG, kAlt>(Q, P.c, A);
  const T qd = ld_sol<kCG>(Q + P.d), qe = ld_sol<kCG>(Q + P.e);
  const T g = P.g >= 0 ? bcg[P.g] : T(0);
  return ghost_formula<T>(P.ty, qa, qb, qc, qd, qe, g, P.nb, hx, hy);
}

template <class T, bool kCG = false, bool kAlt = false>
__device__ __forceinline__ void ghost_apply(const GhostItems &G, int i, const GhostPrep &P, T *Q, T *QC, const T *bcg,
                                            T hx, T hy, const GhostAlt *A = nullptr) {
  if (P.ty == G_PHYS_CORNER) {
    if (!kAlt) {
      ghost_item<T, kCG>(G, i, P.ty, P.dst, Q, QC, bcg, hx, hy);
      return;
    }
    // (face ghost 1 + face ghost 2) - interior, each face ghost by its own
    // rule with the fused fill's operands
    const int r1 = G.a[i], r2 = G.b[i];
    const T v1 = ghost_value<T, kCG, true>(ghost_prep<true>(G, r1, G.type[r1], 0, A), Q, bcg, hx, hy, A);
    const T v2 = ghost_value<T, kCG, true>(ghost_prep<true>(G, r2, G.type[r2], 0, A), Q, bcg, hx, hy, A);
    Q[P.dst] = (v1 + v2) - ghost_operand<T, kCG, true>(Q, __ldg(A->c + i), A);
    return;
  }
  if (P.ty == G_RING) {
    QC[P.dst] = ld_sol<kCG>(Q + P.a);
    return;
  }
  Q[P.dst] = ghost_value<T, kCG, kAlt>(P, Q, bcg, hx, hy, A);
}

// kT threads per block: kBlock, or 64 on a level whose kBlock grid leaves
// SMs idle
template <class T, int kT = kBlock>
__global__ void __launch_bounds__(kT) k_ghost(GhostItems G, int off, int n, T *__restrict__ Q, T *__restrict__ QC,
                                              const T *__restrict__ bcg, double hx_, double hy_,
                                              const int *__restrict__ active, const int *__restrict__ inst_nlev,
                                              int need) {
  chain_trigger();
  const int t = blockIdx.x * kT + threadIdx.x;
  const int i = off + t;
  // a converged instance of a batch stays frozen; a fill that follows the
  // restriction from level `need` skips the instances without that level
  // (their own V-cycle starts below it)
  const int inst = (t < n && G.inst) ? G.inst[i] : -1;
  const bool skip = t >= n || (inst >= 0 && (!active[inst] || inst_nlev[inst] < need));
  GhostPrep P;
  if (!skip) P = ghost_prep(G, i, G.type[i], G.dst[i]);
  chain_wait();
  if (skip) return;
  ghost_apply<T>(G, i, P, Q, QC, bcg, T(hx_), T(hy_));
}

// Ghost fills of several levels in one launch: span s holds the items
// [off[s], off[s] + beg[s+1] - beg[s]) of a level with cell sizes hx[s],
// hy[s], and launch item t belongs to the span with beg[s] <= t < beg[s+1].
// The host groups levels none of which reads a ghost cell that another level
// of the launch writes.
constexpr int kMaxSpans = 16;
struct GhostSpans {
  int off[kMaxSpans], beg[kMaxSpans + 1];
  double hx[kMaxSpans], hy[kMaxSpans];
  int n;
};

template <class T, int kT = kBlock>
__global__ void __launch_bounds__(kT) k_ghost_spans(GhostItems G, GhostSpans S, T *__restrict__ Q,
                                                    T *__restrict__ QC, const T *__restrict__ bcg,
                                                    const int *__restrict__ active) {
  chain_trigger();
  const int t = blockIdx.x * kT + threadIdx.x;
  int off = S.off[0], b = 0, tot = 0;
  double hx = S.hx[0], hy = S.hy[0];
#pragma unroll
  for (int j = 1; j <= kMaxSpans; ++j) {
    if (j == S.n) tot = S.beg[j];
    if (j < kMaxSpans && j < S.n && t >= S.beg[j]) {
      off = S.off[j];
      b = S.beg[j];
      hx = S.hx[j];
      hy = S.hy[j];
    }
  }
  const bool in = t < tot;
  const int i = off + (t - b);
  const int inst = (in && G.inst) ? G.inst[i] : -1;
  const bool skip = !in || (inst >= 0 && !active[inst]);
  GhostPrep P;
  if (!skip) P = ghost_prep(G, i, G.type[i], G.dst[i]);
  chain_wait();
  if (skip) return;
  ghost_apply<T>(G, i, P, Q, QC, bcg, T(hx), T(hy));
}

// ---------------------------------------------------------------------------
// relax2d (EllipticBSAM/src/ebKernels.m:37-95): one colour of the red-black
// Gauss-Seidel sweep over all patches of a level, one thread per cell of
// the colour.  The colour cells of each patch are cut into chunks of
// kChunk that never straddle two patches; a chunk record carries everything
// a thread needs about its patch, so one load precedes the data loads.
// Partial physical ghosts ((8/3)g + (1/3)u_2 Dirichlet, h g Neumann) are
// formed in registers, the u_1 coupling being folded into InvDiagS.  The
// reference refills every ghost after each colour (ebRelaxLevel.m:36); with
// `fresh` set, a boundary thread instead evaluates its neighbour ghost's
// rule (stored inline per perimeter cell): every rule of an internal face
// reads only cells of the other colour (final after the previous pass),
// parent cells, or the reading cell itself (pre-update), so the value equals
// the refilled ghost bit for bit.  The first pass of a relaxation reads the
// ghosts as the last fill left them, as the reference does.
constexpr int kChunk = 64;

struct RelaxChunk {           // host record (packing of the operands)
  int q_off, c_off, dew_off, dns_off;
  int bcg_off, pe_off, mx, my;
  int par0, s0, n, inst;     // first colour-cell index in the patch, cells in the chunk, instance
  int bc[4];
};

// the chunk as the smoother kernels read it: three 16-byte words (three
// vector loads, ten registers); flags holds the W, E, S, N boundary codes in
// 2-bit fields and par0 in bit 8
struct __align__(16) RelaxChunkD {
  int q_off, c_off, bcg_off, pe_off;
  int mx, my, s0, n;
  int inst, flags, pad0, pad1;
};

// how a smoother chunk learns that its instance is frozen: kActNone, one
// instance (always live while a V-cycle runs); kActChunk, the per-chunk flag
// array k_residual_final keeps (a batch's instances' chunks are contiguous
// per level)
enum { kActNone = 0, kActChunk = 1 };

__device__ __forceinline__ int chunk_bc(int flags, int side) { return (flags >> (2 * side)) & 3; }
__device__ __forceinline__ int chunk_par0(int flags) { return (flags >> 8) & 1; }

// one ghost rule, inline (perimeter table): 32 bytes, two vector loads.  The
// operand slots a rule does not use repeat its first operand (set at
// upload), so all five can be read whatever the rule's kind.
struct __align__(16) Rule {
  int type, a, b, c, d, e, pad0, pad1;
};

// Every operand is requested before the rule's kind is looked at: the lanes
// of a warp that evaluate different kinds of rules then wait for one round of
// loads together, instead of one dependent round per kind in turn (the
// divergent branches would otherwise serialise their load latencies).
template <class T, bool kCG = false>
__device__ __forceinline__ T eval_inline(const Rule &R, const T *Q) {
  const T qa = ld_sol<kCG>(Q + R.a), qb = ld_sol<kCG>(Q + R.b), qc = ld_sol<kCG>(Q + R.c);
  const T qd = ld_sol<kCG>(Q + R.d), qe = ld_sol<kCG>(Q + R.e);
  return rule_value<T>(R.type, qa, qb, qc, qd, qe);
}

// The smoother's operands per chunk and colour, packed at upload: for chunk
// ch and colour m, five rows of kChunk values -- dE, dW, dN, dS (pre-scaled
// by 1/h^2 on power-of-two levels) and InvDiagS -- one per colour cell of
// the chunk, so a warp reads each operand as one contiguous row instead of
// every other value of the reference's arrays.
constexpr int kPackRows = 5;

// a static table row (never written while kernels run) brought into L1
// before the programmatic-launch wait; the read after the wait then hits L1
// without holding the row in registers across the wait
template <class R>
__device__ __forceinline__ void prefetch_l1(const R *p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
  asm volatile("prefetch.global.L1 [%0];" ::"l"((const char *)(p + 1) - 1));
}

// Builds the packed operands of one level's chunks on the device from the
// reference-layout DeW, DnS and InvDiagS (one thread per chunk, colour and
// slot; slots past a chunk's cell count are zero).  `scale` multiplies the
// face coefficients by the exact 1/h^2 of a power-of-two level (ix, iy), the
// same product the relaxation's pre-scaled form relies on.
__global__ void __launch_bounds__(kBlock) k_pack(const RelaxChunk *__restrict__ ch, int nch,
                                                 const double *__restrict__ DeW, const double *__restrict__ DnS,
                                                 const double *__restrict__ ID, double ix, double iy, int scale,
                                                 double *__restrict__ pack) {
  const int64_t w = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (w >= (int64_t)nch * 2 * kChunk) return;
  const int c = (int)(w / (2 * kChunk)), m = (int)((w / kChunk) & 1), t = (int)(w % kChunk);
  const RelaxChunk R = ch[c];
  double *o = pack + ((size_t)c * 2 + m) * (kPackRows * kChunk) + t;
  if (t >= R.n) {
#pragma unroll
    for (int r = 0; r < kPackRows; ++r) o[r * kChunk] = 0.0;
    return;
  }
  const int s = R.s0 + t, half = R.mx >> 1;
  const int lj = s / half;
  const int li = 2 * (s - lj * half) + ((m + lj + R.par0) & 1);
  double e = DeW[R.dew_off + (li + 1) + lj * (R.mx + 1)], wv = DeW[R.dew_off + li + lj * (R.mx + 1)];
  double n = DnS[R.dns_off + li + (lj + 1) * R.mx], sv = DnS[R.dns_off + li + lj * R.mx];
  if (scale) {
    e = e * ix;
    wv = wv * ix;
    n = n * iy;
    sv = sv * iy;
  }
  o[0] = e;
  o[kChunk] = wv;
  o[2 * kChunk] = n;
  o[3 * kChunk] = sv;
  o[4 * kChunk] = ID[R.c_off + li + lj * R.mx];
}

// One colour-cell update in three stages, so that a persistent block can
// overlap them across chunk groups (k_relax_p): issue (the chunk record, its
// frozen flag and the packed operands), derive (the cell's position, its
// boundary data and ghost rules, all static), update (solution loads, ghost
// values, the candidate and its store).  relax_cell runs the three in order.
template <class T>
struct CellState {
  RelaxChunkD R;
  T dE, dW, dN, dS, idg, gx, gy;
  int q_off, c, cc, ldq, code, rx, ry;   // code: kx | ky << 2 | sx << 4 | sy << 5
  bool live;
};

// the chunk record, its frozen flag and the packed operands are indexed by
// the chunk alone: record and flag are requested together, the operands (a
// chunk's pack rows hold kChunk entries whatever its cell count) as soon as
// the small, cached flag says the chunk is live, so they are in flight with
// the record and a frozen chunk reads nothing else
template <class T>
__device__ __forceinline__ void cell_issue(const RelaxChunkD *__restrict__ chunks, int nchunks,
                                           const T *__restrict__ pack, int m, const uint8_t *__restrict__ cact,
                                           int amode, int ch, int tc, CellState<T> &S) {
  const bool okc = ch < nchunks;
  S.live = okc;
  S.dE = S.dW = S.dN = S.dS = S.idg = T(0);
  if (okc) {
    S.R = chunks[ch];
    if (amode == kActChunk) S.live = cact[ch] != 0;
  }
  if (S.live) {
    const T *__restrict__ pk = pack + (size_t)(ch * 2 + m) * (kPackRows * kChunk) + tc;
    S.dE = __ldg(pk);
    S.dW = __ldg(pk + kChunk);
    S.dN = __ldg(pk + 2 * kChunk);
    S.dS = __ldg(pk + 3 * kChunk);
    S.idg = __ldg(pk + 4 * kChunk);
  }
}

template <class T>
__device__ __forceinline__ void cell_derive(const FieldsT<T> &f, const Rule *__restrict__ perim, int m, int fresh,
                                            int tc, CellState<T> &S) {
  if (!S.live || tc >= S.R.n) {
    S.live = false;
    return;
  }
  const RelaxChunkD &R = S.R;
  const int s = R.s0 + tc;
  const int mx = R.mx, my = R.my, half = mx >> 1;
  const int lj = s / half;
  const int li = 2 * (s - lj * half) + ((m + lj + chunk_par0(R.flags)) & 1);
  S.ldq = mx + 2;
  S.c = (li + 1) + (lj + 1) * S.ldq;
  S.cc = R.c_off + li + lj * mx;
  S.q_off = R.q_off;
  // static boundary data and ghost rules; a cell touches at most one x side
  // (W or E) and one y side (S or N): kind 0 interior neighbour, 1
  // Dirichlet, 2 Neumann, 3 ghost rule
  const T *__restrict__ g4 = f.bcg + R.bcg_off;
  int kx = 0, ky = 0, sx = 0, sy = 0;       // sx: 0 west 1 east; sy: 0 south 1 north
  S.gx = S.gy = T(0);
  S.rx = S.ry = 0;                          // ghost rule indices (perimeter table)
  if (li == 0 || li == mx - 1) {
    sx = (li == 0) ? 0 : 1;
    const int bc = chunk_bc(R.flags, sx);   // a shift, not an indexed (local-memory) array
    if (bc) { kx = bc; S.gx = __ldg(g4 + sx * my + lj); }
    else if (fresh) { kx = 3; S.rx = R.pe_off + sx * my + lj; prefetch_l1(perim + S.rx); }
  }
  if (lj == 0 || lj == my - 1) {
    sy = (lj == 0) ? 0 : 1;
    const int bc = chunk_bc(R.flags, 2 + sy);
    if (bc) { ky = bc; S.gy = __ldg(g4 + 2 * my + sy * mx + li); }
    else if (fresh) { ky = 3; S.ry = R.pe_off + 2 * my + sy * mx + li; prefetch_l1(perim + S.ry); }
  }
  S.code = kx | (ky << 2) | (sx << 4) | (sy << 5);
}

template <class T, bool kPow2, bool kCG>
__device__ __forceinline__ void cell_update(const LevelD &L, const FieldsT<T> &f, const Rule *__restrict__ perim,
                                            T omega, int unit_omega, const CellState<T> &S) {
  if (!S.live) return;
  const T c83 = T(8.0 / 3.0), c13 = T(1.0 / 3.0);
  const LevelH<T> H = level_h(L, T(0));
  const int c = S.c, ldq = S.ldq;
  const int kx = S.code & 3, ky = (S.code >> 2) & 3, sx = (S.code >> 4) & 1, sy = (S.code >> 5) & 1;
  T *__restrict__ Q = f.Q + S.q_off;
  T qe = ld_sol<kCG>(Q + c + 1), qw = ld_sol<kCG>(Q + c - 1), qn = ld_sol<kCG>(Q + c + ldq), qs = ld_sol<kCG>(Q + c - ldq);
  T t = f.F[S.cc];
  // the operands of the neighbour ghost's rule are requested with the
  // solution loads, before any value is formed, so lanes with different kinds
  // of ghosts wait for a single round of loads.  A lane holds one rule's
  // operands: a patch-corner cell with rules on both sides (x and y) forms
  // its y-side ghost in a second round.
  const bool rx = kx == 3, ry = ky == 3;
  T o0 = T(0), o1 = T(0), o2 = T(0), o3 = T(0), o4 = T(0);
  int rt = 0;
  if (rx || ry) {
    const Rule R = perim[rx ? S.rx : S.ry];
    rt = R.type;
    o0 = ld_sol<kCG>(f.Q + R.a); o1 = ld_sol<kCG>(f.Q + R.b); o2 = ld_sol<kCG>(f.Q + R.c);
    o3 = ld_sol<kCG>(f.Q + R.d); o4 = ld_sol<kCG>(f.Q + R.e);
  }
  // a partial Dirichlet ghost reads the interior neighbour across the cell,
  // which is the opposite neighbour already loaded
  if (kx > 0) {
    T v;
    if (kx == 1) v = c83 * S.gx + c13 * (sx ? qw : qe);
    else if (kx == 2) v = H.hx * S.gx;
    else v = rule_value<T>(rt, o0, o1, o2, o3, o4);
    if (sx) qe = v; else qw = v;
  }
  if (ky > 0) {
    T v;
    if (ky == 1) v = c83 * S.gy + c13 * (sy ? qs : qn);
    else if (ky == 2) v = H.hy * S.gy;
    else if (rx) v = eval_inline<T, kCG>(perim[S.ry], f.Q);
    else v = rule_value<T>(rt, o0, o1, o2, o3, o4);
    if (sy) qn = v; else qs = v;
  }
  // kPow2: the coefficients arrive pre-scaled by the exact 1/h^2 (a power of
  // two), and (q D) 2^-k == q (D 2^-k) in floating point, so one product
  // per neighbour gives the reference's (q D)/h^2 bit for bit
  if (kPow2) {
    t = t + qe * S.dE;
    t = t + qw * S.dW;
    t = t + qn * S.dN;
    t = t + qs * S.dS;
  } else {
    t = t + (qe * S.dE) / H.hx2;
    t = t + (qw * S.dW) / H.hx2;
    t = t + (qn * S.dN) / H.hy2;
    t = t + (qs * S.dS) / H.hy2;
  }
  t = t * S.idg;
  if (unit_omega) Q[c] = t;
  else Q[c] = omega * t + (1 - omega) * ld_sol<kCG>(Q + c);
}

// one colour-cell update of chunk ch (thread tc of the chunk); kChain: the
// grid kernel's programmatic-launch wait sits between the static stages and
// the first read of the solution
template <class T, bool kPow2, bool kChain, bool kCG = false>
__device__ __forceinline__ void relax_cell(const LevelD &L, const RelaxChunkD *__restrict__ chunks, int nchunks,
                                           const FieldsT<T> &f, const T *__restrict__ pack,
                                           const Rule *__restrict__ perim, int m, T omega, int unit_omega, int fresh,
                                           const uint8_t *__restrict__ cact, int amode, int ch, int tc) {
  CellState<T> S;
  cell_issue<T>(chunks, nchunks, pack, m, cact, amode, ch, tc, S);
  cell_derive<T>(f, perim, m, fresh, tc, S);
  if (kChain) chain_wait();
  cell_update<T, kPow2, kCG>(L, f, perim, omega, unit_omega, S);
}

// Persistent form of one colour pass: a grid of resident blocks walks the
// level's chunk groups (kBlock / kChunk chunks each) with a grid stride;
// while a block updates one group it has the next group's chunk records and
// operands in flight, and derives that group's static data after the
// update.  The arithmetic of every update is relax_cell's.
template <class T, bool kPow2>
__global__ void __launch_bounds__(kBlock) k_relax_p(LevelD L, const RelaxChunkD *__restrict__ chunks, int nchunks,
                                                    FieldsT<T> f, const T *__restrict__ pack,
                                                    const Rule *__restrict__ perim, int m, T omega, int unit_omega,
                                                    int fresh, const uint8_t *__restrict__ cact, int amode) {
  chain_trigger();
  constexpr int cpb = kBlock / kChunk;
  const int sub = threadIdx.x / kChunk, tc = threadIdx.x & (kChunk - 1);
  const int ngroups = (nchunks + cpb - 1) / cpb;
  int g = blockIdx.x;
  CellState<T> cur, nxt;
  cell_issue<T>(chunks, nchunks, pack, m, cact, amode, g * cpb + sub, tc, cur);
  cell_derive<T>(f, perim, m, fresh, tc, cur);
  chain_wait();
  while (g < ngroups) {
    const int gn = g + (int)gridDim.x;
    cell_issue<T>(chunks, nchunks, pack, m, cact, amode, gn * cpb + sub, tc, nxt);
    cell_update<T, kPow2, false>(L, f, perim, omega, unit_omega, cur);
    cell_derive<T>(f, perim, m, fresh, tc, nxt);
    cur = nxt;
    g = gn;
  }
}

// Coarsened smoother: each thread updates kN colour cells of its chunk
// (cells t, t + kChunk/kN, ...), in three phases -- static loads of every
// cell, then the solution loads of every cell, then every update -- so the
// loads of a thread's cells are in flight together.  Within a colour pass no
// cell reads another cell of its colour (a ghost rule reads cells of the
// other colour, parent cells or the reading cell itself, before its update),
// so loading all before storing any changes nothing: the arithmetic of each
// update is relax_cell's.
template <class T, bool kPow2, int kN>
__global__ void __launch_bounds__(kBlock) k_relax_n(LevelD L, const RelaxChunkD *__restrict__ chunks, int nchunks,
                                                    FieldsT<T> f, const T *__restrict__ pack,
                                                    const Rule *__restrict__ perim, int m, T omega, int unit_omega,
                                                    int fresh, const uint8_t *__restrict__ cact, int amode) {
  chain_trigger();
  constexpr int tpc = kChunk / kN;                    // threads per chunk
  const int ch = blockIdx.x * (kBlock / tpc) + threadIdx.x / tpc;
  const int t0 = threadIdx.x % tpc;
  // chunk record and packed operands requested together (as relax_cell)
  const bool okc = ch < nchunks;
  RelaxChunkD R;
  bool live = okc;
  T dE[kN], dW[kN], dN[kN], dS[kN], idg[kN], gx[kN], gy[kN];
  if (okc) {
    R = chunks[ch];
    if (amode == kActChunk) live = cact[ch] != 0;
  }
  if (live) {
    const T *__restrict__ pk0 = pack + (size_t)(ch * 2 + m) * (kPackRows * kChunk) + t0;
#pragma unroll
    for (int u = 0; u < kN; ++u) {
      const T *__restrict__ pk = pk0 + u * tpc;
      dE[u] = __ldg(pk);
      dW[u] = __ldg(pk + kChunk);
      dN[u] = __ldg(pk + 2 * kChunk);
      dS[u] = __ldg(pk + 3 * kChunk);
      idg[u] = __ldg(pk + 4 * kChunk);
    }
  }
  if (!live || t0 >= R.n) {
    chain_wait();
    return;
  }
  const int mx = R.mx, my = R.my, half = mx >> 1, ldq = mx + 2;
  const T *__restrict__ g4 = f.bcg + R.bcg_off;
  bool on[kN];
  int c[kN], cc[kN], code[kN], rxi[kN], ryi[kN];    // code: kx | ky << 2 | sx << 4 | sy << 5
#pragma unroll
  for (int u = 0; u < kN; ++u) {
    const int tc = t0 + u * tpc;
    on[u] = tc < R.n;
    const int s = R.s0 + (on[u] ? tc : 0);
    const int lj = s / half;
    const int li = 2 * (s - lj * half) + ((m + lj + chunk_par0(R.flags)) & 1);
    c[u] = (li + 1) + (lj + 1) * ldq;
    cc[u] = R.c_off + li + lj * mx;
    int kx = 0, ky = 0, sx = 0, sy = 0;
    gx[u] = 0;
    gy[u] = 0;
    rxi[u] = 0;
    ryi[u] = 0;
    if (li == 0 || li == mx - 1) {
      sx = (li == 0) ? 0 : 1;
      const int bc = chunk_bc(R.flags, sx);
      if (bc) { kx = bc; gx[u] = __ldg(g4 + sx * my + lj); }
      else if (fresh) { kx = 3; rxi[u] = R.pe_off + sx * my + lj; prefetch_l1(perim + rxi[u]); }
    }
    if (lj == 0 || lj == my - 1) {
      sy = (lj == 0) ? 0 : 1;
      const int bc = chunk_bc(R.flags, 2 + sy);
      if (bc) { ky = bc; gy[u] = __ldg(g4 + 2 * my + sy * mx + li); }
      else if (fresh) { ky = 3; ryi[u] = R.pe_off + 2 * my + sy * mx + li; prefetch_l1(perim + ryi[u]); }
    }
    code[u] = kx | (ky << 2) | (sx << 4) | (sy << 5);
  }
  chain_wait();
  const T c83 = T(8.0 / 3.0), c13 = T(1.0 / 3.0);
  const LevelH<T> H = level_h(L, T(0));
  T *__restrict__ Q = f.Q + R.q_off;
  T qe[kN], qw[kN], qn[kN], qs[kN], fv[kN], qc[kN];
#pragma unroll
  for (int u = 0; u < kN; ++u) {
    const int cu = c[u];
    qe[u] = Q[cu + 1];
    qw[u] = Q[cu - 1];
    qn[u] = Q[cu + ldq];
    qs[u] = Q[cu - ldq];
    qc[u] = unit_omega ? T(0) : Q[cu];
    fv[u] = f.F[cc[u]];
  }
#pragma unroll
  for (int u = 0; u < kN; ++u) {
    const int kx = code[u] & 3, ky = (code[u] >> 2) & 3, sx = (code[u] >> 4) & 1, sy = (code[u] >> 5) & 1;
    const int cu = c[u];
    if (kx > 0) {
      T v;
      if (kx == 1) v = c83 * gx[u] + c13 * Q[sx ? cu - 1 : cu + 1];
      else if (kx == 2) v = H.hx * gx[u];
      else v = eval_inline<T>(perim[rxi[u]], f.Q);
      if (sx) qe[u] = v; else qw[u] = v;
    }
    if (ky > 0) {
      T v;
      if (ky == 1) v = c83 * gy[u] + c13 * Q[sy ? cu - ldq : cu + ldq];
      else if (ky == 2) v = H.hy * gy[u];
      else v = eval_inline<T>(perim[ryi[u]], f.Q);
      if (sy) qn[u] = v; else qs[u] = v;
    }
  }
#pragma unroll
  for (int u = 0; u < kN; ++u) {
    if (!on[u]) continue;
    T t = fv[u];
    if (kPow2) {
      t = t + qe[u] * dE[u];
      t = t + qw[u] * dW[u];
      t = t + qn[u] * dN[u];
      t = t + qs[u] * dS[u];
    } else {
      t = t + (qe[u] * dE[u]) / H.hx2;
      t = t + (qw[u] * dW[u]) / H.hx2;
      t = t + (qn[u] * dN[u]) / H.hy2;
      t = t + (qs[u] * dS[u]) / H.hy2;
    }
    t = t * idg[u];
    if (unit_omega) Q[c[u]] = t;
    else Q[c[u]] = omega * t + (1 - omega) * qc[u];
  }
}

// kT threads per block: kBlock, or kChunk (one chunk per block) on a level
// whose kBlock grid would leave SMs idle -- an SM issues about two FP64
// operations per clock, so a block's FP64 work is spread over more SMs
// (same arithmetic, same register budget per thread)
template <class T, bool kPow2, int kT = kBlock>
__global__ void __launch_bounds__(kT, (sizeof(T) == 4 ? 8 : 5) * (kBlock / kT))
    k_relax(LevelD L, const RelaxChunkD *__restrict__ chunks, int nchunks, FieldsT<T> f, const T *__restrict__ pack,
            const Rule *__restrict__ perim, int m, T omega, int unit_omega, int fresh,
            const uint8_t *__restrict__ cact, int amode) {
  chain_trigger();
  relax_cell<T, kPow2, true>(L, chunks, nchunks, f, pack, perim, m, omega, unit_omega, fresh, cact, amode,
                             blockIdx.x * (kT / kChunk) + threadIdx.x / kChunk, threadIdx.x & (kChunk - 1));
}

// A small level's whole relaxation in one launch: one thread-block cluster
// runs every colour pass of the `nsweeps` sweeps over all the level's chunks
// (cluster-strided), with a cluster barrier (release / acquire) between
// passes, then the level's ghost fill (launch_fill's items).  Each pass and
// the fill compute exactly what the separate launches compute -- the same
// relax_cell and ghost_apply code -- with the solution read from L2.  One
// cluster holds every block, so the barrier orders the whole level; no
// thread leaves the loop early, so every barrier is reached by all.
constexpr int kClusterBlock = 1024;

template <class T, bool kPow2>
__global__ void __launch_bounds__(kClusterBlock, 1)
    k_relax_cluster(LevelD L, const RelaxChunkD *__restrict__ chunks, int nchunks, FieldsT<T> f,
                    const T *__restrict__ pack, const Rule *__restrict__ perim, T omega, int unit_omega, int nsweeps,
                    int first_fresh, const uint8_t *__restrict__ cact, int amode, GhostItems G, int g_off, int g_n,
                    double hx_, double hy_) {
  namespace cg = cooperative_groups;
  chain_trigger();
  cg::cluster_group cl = cg::this_cluster();
  const int nth = (int)cl.num_blocks() * kClusterBlock;
  const int tid = (int)cl.block_rank() * kClusterBlock + threadIdx.x;
  chain_wait();
  const int nitems = nchunks * kChunk;
  for (int s = 0; s < nsweeps; ++s)
    for (int m = 0; m < 2; ++m) {
      const int fresh = (first_fresh || s > 0 || m > 0) ? 1 : 0;
      for (int w = tid; w < nitems; w += nth)
        relax_cell<T, kPow2, false, true>(L, chunks, nchunks, f, pack, perim, m, omega, unit_omega, fresh, cact,
                                          amode, w / kChunk, w % kChunk);
      cl.sync();
    }
  for (int t = tid; t < g_n; t += nth) {
    const int i = g_off + t;
    const int inst = G.inst ? G.inst[i] : -1;
    if (inst >= 0 && !f.active[inst]) continue;
    ghost_apply<T, true>(G, i, ghost_prep(G, i, G.type[i], G.dst[i]), f.Q, f.QC, f.bcg, T(hx_), T(hy_));
  }
}


// A small level's relaxation with its solution in distributed shared
// memory.  One thread-block cluster copies the level's Q range [q0, q0 + qn)
// into the shared memory of its CTAs (CTA r holds elements [r S, (r + 1) S),
// S = 2^shift), runs every colour pass of the `nsweeps` sweeps with the
// neighbour and ghost-rule loads and the stores going to the owning CTA's
// shared memory, a cluster barrier between passes, then the level's ghost
// fill (g_n > 0), and copies the range back.  Each thread owns one chunk
// slot (the same colour-cell position of both colours) and loads its static
// data once, before the passes: the packed operands, boundary data, force,
// and its ghost rule with the rule's parent-cell operands (cells outside the
// range do not change during the relaxation), so a pass waits only for the
// shared-memory loads of the solution.  The arithmetic of every update and
// ghost is relax_cell's and ghost_item's, so the results are the chained
// passes' bit for bit.  The host uses it on levels with at most one colour
// cell per thread and colour; the dynamic shared memory is the slice and
// ten values per thread (the rules' parent-cell operands).
constexpr int kDsmBlock = 512;   // threads per CTA of k_relax_dsm

template <class T>
struct DsmRange {
  int q0, qn, shift;
  uint32_t base;          // shared-window address of this CTA's slice
};

template <class T>
__device__ __forceinline__ uint32_t dsm_addr(const DsmRange<T> &D, int rel) {
  const uint32_t la = D.base + (uint32_t)(rel & ((1 << D.shift) - 1)) * (uint32_t)sizeof(T);
  uint32_t ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(la), "r"((uint32_t)rel >> D.shift));
  return ra;
}
__device__ __forceinline__ double dsm_ld(uint32_t a, double) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ float dsm_ld(uint32_t a, float) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ void dsm_st(uint32_t a, double v) {
  asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
}
__device__ __forceinline__ void dsm_st(uint32_t a, float v) {
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}

// a solution value: from the cluster's copy inside the range, else from
// global memory (static while the kernel runs)
template <class T>
__device__ __forceinline__ T dsm_sol(const DsmRange<T> &D, const T *Q, int n) {
  const int rel = n - D.q0;
  if ((unsigned)rel < (unsigned)D.qn) return dsm_ld(dsm_addr(D, rel), T(0));
  return __ldg(Q + n);
}

template <class T>
__device__ __forceinline__ T dsm_rule(const DsmRange<T> &D, const Rule &R, const T *Q) {
  const T qa = dsm_sol(D, Q, R.a), qb = dsm_sol(D, Q, R.b), qc = dsm_sol(D, Q, R.c);
  const T qd = dsm_sol(D, Q, R.d), qe = dsm_sol(D, Q, R.e);
  return rule_value<T>(R.type, qa, qb, qc, qd, qe);
}

// one colour cell's static data for k_relax_dsm; its ghost rule's operands
// outside the range (static) wait in the CTA's shared memory at `ov`
template <class T>
struct DsmCell {
  T dE, dW, dN, dS, idg, gx, gy, fv;
  uint32_t oa[5];        // per rule operand: its shared-window address (inside the range) or global index
  int c, ldq, code, cc, rx, ry, rtype, omask;   // c relative to q0; omask bit i: operand i inside the range
  bool live;
};

// the static part, before the programmatic-launch wait: the cell's packed
// operands and boundary data, and its ghost rule -- kind, and per operand
// the shared-window address (inside the range, mask bit set) or the global
// index whose value the bind loads
template <class T>
__device__ __forceinline__ void dsm_cell_static(const RelaxChunkD *__restrict__ chunks, int nchunks,
                                                const T *__restrict__ pack, const FieldsT<T> &f,
                                                const Rule *__restrict__ perim, const uint8_t *__restrict__ cact,
                                                int amode, int ch, int tc, int m, const DsmRange<T> &D,
                                                DsmCell<T> &X) {
  CellState<T> S;
  cell_issue<T>(chunks, nchunks, pack, m, cact, amode, ch, tc, S);
  cell_derive<T>(f, perim, m, 1, tc, S);
  X.live = S.live;
  X.dE = S.dE; X.dW = S.dW; X.dN = S.dN; X.dS = S.dS; X.idg = S.idg; X.gx = S.gx; X.gy = S.gy;
  X.c = S.q_off + S.c - D.q0;
  X.ldq = S.ldq;
  X.code = S.code;
  X.cc = S.cc;
  X.rx = S.rx;
  X.ry = S.ry;
  X.rtype = 0;
  X.omask = 0;
  const int kx = X.code & 3, ky = (X.code >> 2) & 3;
  if (X.live && (kx == 3 || ky == 3)) {
    const Rule R = perim[kx == 3 ? X.rx : X.ry];
    X.rtype = R.type;
    const int op[5] = {R.a, R.b, R.c, R.d, R.e};
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const int rel = op[i] - D.q0;
      if ((unsigned)rel < (unsigned)D.qn) {
        X.omask |= 1 << i;
        X.oa[i] = dsm_addr(D, rel);
      } else {
        X.oa[i] = (uint32_t)op[i];
      }
    }
  }
}

// the dynamic part of the set-up, after the wait: the force and the values
// of the rule's operands outside the range (into ov)
template <class T>
__device__ __forceinline__ void dsm_cell_bind(const FieldsT<T> &f, T *ov, DsmCell<T> &X) {
  if (!X.live) return;
  X.fv = f.F[X.cc];
  const int kx = X.code & 3, ky = (X.code >> 2) & 3;
  if (kx == 3 || ky == 3) {
#pragma unroll
    for (int i = 0; i < 5; ++i)
      if (!((X.omask >> i) & 1)) ov[i] = f.Q[(int)X.oa[i]];
  }
}

// cell_update from the static data and the cluster's copy of the solution
template <class T, bool kPow2>
__device__ __forceinline__ void dsm_cell_update(const LevelD &L, const FieldsT<T> &f, const Rule *__restrict__ perim,
                                                T omega, int unit_omega, int fresh, const DsmCell<T> &X,
                                                const T *ov, const DsmRange<T> &D) {
  if (!X.live) return;
  const T c83 = T(8.0 / 3.0), c13 = T(1.0 / 3.0);
  const LevelH<T> H = level_h(L, T(0));
  const int ldq = X.ldq, c = X.c;
  int kx = X.code & 3, ky = (X.code >> 2) & 3;
  const int sx = (X.code >> 4) & 1, sy = (X.code >> 5) & 1;
  if (!fresh) {               // the stored ghosts, as the last fill left them
    if (kx == 3) kx = 0;
    if (ky == 3) ky = 0;
  }
  T qe = dsm_ld(dsm_addr(D, c + 1), T(0)), qw = dsm_ld(dsm_addr(D, c - 1), T(0));
  T qn = dsm_ld(dsm_addr(D, c + ldq), T(0)), qs = dsm_ld(dsm_addr(D, c - ldq), T(0));
  T t = X.fv;
  const bool rx = kx == 3, ry = ky == 3;
  T o[5];
#pragma unroll
  for (int i = 0; i < 5; ++i)
    o[i] = (rx || ry) ? (((X.omask >> i) & 1) ? dsm_ld(X.oa[i], T(0)) : ov[i]) : T(0);
  if (kx > 0) {
    T v;
    if (kx == 1) v = c83 * X.gx + c13 * (sx ? qw : qe);
    else if (kx == 2) v = H.hx * X.gx;
    else v = rule_value<T>(X.rtype, o[0], o[1], o[2], o[3], o[4]);
    if (sx) qe = v; else qw = v;
  }
  if (ky > 0) {
    T v;
    if (ky == 1) v = c83 * X.gy + c13 * (sy ? qs : qn);
    else if (ky == 2) v = H.hy * X.gy;
    else if (rx) v = dsm_rule<T>(D, perim[X.ry], f.Q);
    else v = rule_value<T>(X.rtype, o[0], o[1], o[2], o[3], o[4]);
    if (sy) qn = v; else qs = v;
  }
  if (kPow2) {
    t = t + qe * X.dE;
    t = t + qw * X.dW;
    t = t + qn * X.dN;
    t = t + qs * X.dS;
  } else {
    t = t + (qe * X.dE) / H.hx2;
    t = t + (qw * X.dW) / H.hx2;
    t = t + (qn * X.dN) / H.hy2;
    t = t + (qs * X.dS) / H.hy2;
  }
  t = t * X.idg;
  const uint32_t ac = dsm_addr(D, c);
  if (unit_omega) dsm_st(ac, t);
  else dsm_st(ac, omega * t + (1 - omega) * dsm_ld(ac, T(0)));
}

// one ghost rule's value (eval_rule's arithmetic) from the cluster's copy
template <class T>
__device__ __forceinline__ T ghost_eval_dsm(const GhostItems &G, int i, const FieldsT<T> &f, T hx, T hy,
                                            const DsmRange<T> &D) {
  const GhostPrep P = ghost_prep(G, i, G.type[i], 0);
  const T qa = dsm_sol(D, f.Q, P.a), qb = dsm_sol(D, f.Q, P.b), qc = dsm_sol(D, f.Q, P.c);
  const T qd = dsm_sol(D, f.Q, P.d), qe = dsm_sol(D, f.Q, P.e);
  const T g = P.g >= 0 ? f.bcg[P.g] : T(0);
  return ghost_formula<T>(P.ty, qa, qb, qc, qd, qe, g, P.nb, hx, hy);
}

template <class T, bool kPow2>
__global__ void __launch_bounds__(kDsmBlock, 1)
    k_relax_dsm(LevelD L, const RelaxChunkD *__restrict__ chunks, int nchunks, FieldsT<T> f,
                const T *__restrict__ pack, const Rule *__restrict__ perim, T omega, int unit_omega, int nsweeps,
                int first_fresh, const uint8_t *__restrict__ cact, int amode, GhostItems G, int g_off, int g_n,
                double hx_, double hy_, int q0, int qn, int shift) {
  namespace cg = cooperative_groups;
  constexpr int kB = kDsmBlock;
  extern __shared__ __align__(16) unsigned char dsm_raw[];
  T *slice = reinterpret_cast<T *>(dsm_raw);
  chain_trigger();
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks(), r = (int)cl.block_rank();
  const int S = 1 << shift;
  const DsmRange<T> D{q0, qn, shift, (uint32_t)__cvta_generic_to_shared(slice)};
  // this thread's chunk slot: CTA r takes a contiguous run of chunks
  const int cpc = (nchunks + C - 1) / C;
  const int w = r * cpc * kChunk + (int)threadIdx.x;
  const bool mine = (int)threadIdx.x < cpc * kChunk && w < nchunks * kChunk;
  // parent-cell operands of this thread's two rules, after the slice
  T *ov0 = slice + S + 10 * (int)threadIdx.x, *ov1 = ov0 + 5;
  DsmCell<T> X0, X1;
  X0.live = X1.live = false;
  if (mine) {
    dsm_cell_static<T>(chunks, nchunks, pack, f, perim, cact, amode, w / kChunk, w % kChunk, 0, D, X0);
    dsm_cell_static<T>(chunks, nchunks, pack, f, perim, cact, amode, w / kChunk, w % kChunk, 1, D, X1);
  }
  chain_wait();
  const int e0 = r * S, e1 = min(qn, e0 + S);
  for (int e = e0 + (int)threadIdx.x; e < e1; e += kB) slice[e - e0] = f.Q[q0 + e];
  dsm_cell_bind<T>(f, ov0, X0);
  dsm_cell_bind<T>(f, ov1, X1);
  cl.sync();
  for (int s = 0; s < nsweeps; ++s) {
    dsm_cell_update<T, kPow2>(L, f, perim, omega, unit_omega, (first_fresh || s > 0) ? 1 : 0, X0, ov0, D);
    cl.sync();
    dsm_cell_update<T, kPow2>(L, f, perim, omega, unit_omega, 1, X1, ov1, D);
    cl.sync();
  }
  if (g_n > 0) {
    const int nth = C * kB, tid = r * kB + (int)threadIdx.x;
    const T hx = T(hx_), hy = T(hy_);
    for (int t = tid; t < g_n; t += nth) {
      const int i = g_off + t;
      const int inst = G.inst ? G.inst[i] : -1;
      if (inst >= 0 && !f.active[inst]) continue;
      const int8_t ty = G.type[i];
      const int dst = G.dst[i];
      if (ty == G_RING) {
        f.QC[dst] = dsm_sol(D, f.Q, G.a[i]);
        continue;
      }
      T v;
      if (ty == G_PHYS_CORNER) {
        const T v1 = ghost_eval_dsm<T>(G, G.a[i], f, hx, hy, D);
        const T v2 = ghost_eval_dsm<T>(G, G.b[i], f, hx, hy, D);
        v = (v1 + v2) - dsm_sol(D, f.Q, G.c[i]);
      } else {
        v = ghost_eval_dsm<T>(G, i, f, hx, hy, D);
      }
      dsm_st(dsm_addr(D, dst - q0), v);
    }
    cl.sync();
  }
  for (int e = e0 + (int)threadIdx.x; e < e1; e += kB) f.Q[q0 + e] = slice[e - e0];
}

// ---------------------------------------------------------------------------
// restrict2 (ebKernels.m:98-102) of each patch interior into its QC interior
// and, for 'restrict' (ebTransfer.m:10-33), into the parent's Q over the
// footprint.  One thread per coarse cell.
template <class T>
__device__ __forceinline__ T restrict_cell(const T *Q, int ldq, int ci, int cj) {
  const int c = (2 * ci + 1) + (2 * cj + 1) * ldq;
  return T(0.25) * (((Q[c] + Q[c + 1]) + Q[c + ldq]) + Q[c + ldq + 1]);
}

// one coarse cell of the restriction; kChain: the grid kernel's
// programmatic-launch wait sits between the static loads and the solution
// (every early exit executes it too)
template <class T, bool kChain>
__device__ __forceinline__ void restrict_item(const LevelD &L, const Decomp &D, const FieldsT<T> &f, int to_parent,
                                              int g) {
  if (g >= D.n) {
    if (kChain) chain_wait();
    return;
  }
  const int p = find_patch(D, g / kBlock, g);
  const PatchD &P = L.patches[p];
  if (!f.active[P.inst]) {
    if (kChain) chain_wait();
    return;
  }
  const int cmx = P.mx >> 1, q_off = P.q_off, ldq = P.mx + 2, qc_off = P.qc_off;
  const int s = g - __ldg(D.beg + p);
  const int cj = s / cmx, ci = s - cj * cmx;
  const int dst = to_parent ? __ldg(f.fp + 2 * (P.fp_off + s)) : 0;
  if (kChain) chain_wait();
  const T R = restrict_cell<T>(f.Q + q_off, ldq, ci, cj);
  f.QC[qc_off + (ci + 1) + (cj + 1) * (cmx + 2)] = R;
  if (to_parent) f.Q[dst] = R;
}

// kT threads per block: kBlock, or 64 on a level whose kBlock grid leaves
// SMs idle
template <class T, int kT = kBlock>
__global__ void __launch_bounds__(kT) k_restrict(LevelD L, Decomp D, FieldsT<T> f, int to_parent) {
  chain_trigger();
  restrict_item<T, true>(L, D, f, to_parent, blockIdx.x * kT + threadIdx.x);
}

// The restriction of level k into QC and the parent (ebTransfer.m:10-33)
// and the ghost fill of the parent level that follows it (ebVcycle.m:27,
// ebTransfer.m:73-79) in one launch: blocks [0, nb_r) restrict, the rest
// fill level k-1 with the fused operands of GhostAlt (a fill operand under
// level k's footprint is restricted by the item itself), so no item reads a
// value another item of the launch writes.
//
// Optionally (f_n > 0) the launch also runs level k's own ghost fill that
// precedes the restriction (the closing fill of its pre-smoothing, or of the
// finest level's post-smoothing before the fill-down): blocks
// [nb_r, nb_r + nb_f) run those items as k_ghost does, its ring items only
// with f_ring.  The host allows it on a level whose fill reads no cell the
// restriction or the parent's fill writes, and whose ghost cells the
// parent's fill does not read.  In the FP32 correction cycle it runs on
// every level in the zero-parent form (z_n > 0): the correction starts at 0
// and level k-1 is first written by this very launch, so every parent-level
// operand of level k's pre-smoothing fill is 0, which the items use instead
// of reading cells the launch may be writing.
template <class T, int kT = kBlock>
__global__ void __launch_bounds__(kT) k_restrict_fill(LevelD L, Decomp D, FieldsT<T> f, int to_parent, int nb_r,
                                                     GhostItems G, GhostAlt A, int g_off, int g_n, double hx_,
                                                     double hy_, const int *__restrict__ active,
                                                     const int *__restrict__ inst_nlev, int need, int f_off, int f_n,
                                                     int nb_f, int f_ring, double fhx, double fhy, int z_lo,
                                                     int z_n) {
  chain_trigger();
  if ((int)blockIdx.x < nb_r) {
    restrict_item<T, true>(L, D, f, to_parent, blockIdx.x * kT + threadIdx.x);
    return;
  }
  if ((int)blockIdx.x < nb_r + nb_f) {
    const int t = ((int)blockIdx.x - nb_r) * kT + threadIdx.x;
    const int i = f_off + t;
    const int inst = (t < f_n && G.inst) ? G.inst[i] : -1;
    const int8_t ty = t < f_n ? G.type[i] : G_COPY;
    const bool skip = t >= f_n || (inst >= 0 && !active[inst]) || (ty == G_RING && !f_ring);
    GhostPrep P;
    if (!skip) P = ghost_prep(G, i, ty, G.dst[i]);
    chain_wait();
    if (skip) return;
    if (z_n <= 0) {
      ghost_apply<T>(G, i, P, f.Q, f.QC, f.bcg, T(fhx), T(fhy));
      return;
    }
    // zero-parent form: an operand outside level k's range [z_lo, z_lo + z_n)
    // is a parent-level cell, which holds 0 here (below) -- the value it had
    // before this launch's restriction and parent fill wrote any of them
    const T hx = T(fhx), hy = T(fhy);
    auto op = [&](int n) -> T { return (unsigned)(n - z_lo) < (unsigned)z_n ? f.Q[n] : T(0); };
    auto rule = [&](int j) -> T {
      const GhostPrep R = ghost_prep(G, j, G.type[j], 0);
      return ghost_formula<T>(R.ty, op(R.a), op(R.b), op(R.c), op(R.d), op(R.e), R.g >= 0 ? f.bcg[R.g] : T(0),
                              R.nb, hx, hy);
    };
    if (P.ty == G_PHYS_CORNER) {
      const T v1 = rule(G.a[i]), v2 = rule(G.b[i]);
      f.Q[P.dst] = (v1 + v2) - op(G.c[i]);
    } else {
      f.Q[P.dst] = ghost_formula<T>(P.ty, op(P.a), op(P.b), op(P.c), op(P.d), op(P.e),
                                    P.g >= 0 ? f.bcg[P.g] : T(0), P.nb, hx, hy);
    }
    return;
  }
  const int t = ((int)blockIdx.x - nb_r - nb_f) * kT + threadIdx.x;
  const int i = g_off + t;
  const int inst = (t < g_n && G.inst) ? G.inst[i] : -1;
  const bool skip = t >= g_n || (inst >= 0 && (!active[inst] || inst_nlev[inst] < need));
  GhostPrep P;
  if (!skip) P = ghost_prep<true>(G, i, G.type[i], G.dst[i], &A);
  chain_wait();
  if (skip) return;
  ghost_apply<T, false, true>(G, i, P, f.Q, f.QC, f.bcg, T(hx_), T(hy_), &A);
}
// ---------------------------------------------------------------------------
// ebFaceCorrections (ebFaceCorrections.m:18-61): correction of coarse face j
// on face fc (0 W, 1 E, 2 S, 3 N) of patch P.  The coarse values are read
// where the reference's QC holds them: the outer (ring) cell from the
// parent's Q through the window table, the inner cell from QC's interior
// (`qc_inner` false) or recomputed as the restriction of its four fine cells
// (`qc_inner` true: the residual's refresh, ebCompResidual.m:32-38).
// The arithmetic is FP64 for either value type (the reflux of the mixed
// form stays FP64).
template <class T>
__device__ __forceinline__ double face_corr(const PatchD &P, const FieldsT<T> &f, int fc, int j, double hc2,
                                            double ihc2, int pow2, bool qc_inner) {
  const int mx = P.mx, my = P.my, cmx = mx >> 1, cmy = my >> 1;
  const int ldq = mx + 2, ldc = cmx + 2;
  const T *Q = f.Q + P.q_off, *QC = f.QC + P.qc_off;
  const int *win = f.win + P.win_off;
  const T *DeW = f.DeW + P.dew_off, *DnS = f.DnS + P.dns_off, *cfd = f.cfd + P.cfd_off;
  auto q = [&](int i) { return dbl(Q[i]); };
  double v;
  switch (fc) {
    case 0: {
      const int r1 = 2 * j + 1, r2 = 2 * j + 2;
      const double out = dbl(f.Q[win[(j + 1) * ldc]]);
      const double in = dbl(qc_inner ? restrict_cell<T>(Q, ldq, 0, j) : QC[1 + (j + 1) * ldc]);
      v = (dbl(DeW[(2 * j) * (mx + 1)]) * (q(1 + r1 * ldq) - q(r1 * ldq)) +
           dbl(DeW[(2 * j + 1) * (mx + 1)]) * (q(1 + r2 * ldq) - q(r2 * ldq))) +
          dbl(cfd[j]) * (out - in);
      break;
    }
    case 1: {
      const int r1 = 2 * j + 1, r2 = 2 * j + 2;
      const double out = dbl(f.Q[win[cmx + 1 + (j + 1) * ldc]]);
      const double in = dbl(qc_inner ? restrict_cell<T>(Q, ldq, cmx - 1, j) : QC[cmx + (j + 1) * ldc]);
      v = (dbl(DeW[mx + (2 * j) * (mx + 1)]) * (q(mx + r1 * ldq) - q(mx + 1 + r1 * ldq)) +
           dbl(DeW[mx + (2 * j + 1) * (mx + 1)]) * (q(mx + r2 * ldq) - q(mx + 1 + r2 * ldq))) +
          dbl(cfd[cmy + j]) * (out - in);
      break;
    }
    case 2: {
      const int c1 = 2 * j + 1, c2 = 2 * j + 2;
      const double out = dbl(f.Q[win[j + 1]]);
      const double in = dbl(qc_inner ? restrict_cell<T>(Q, ldq, j, 0) : QC[j + 1 + ldc]);
      v = (dbl(DnS[2 * j]) * (q(c1 + ldq) - q(c1)) + dbl(DnS[2 * j + 1]) * (q(c2 + ldq) - q(c2))) +
          dbl(cfd[2 * cmy + j]) * (out - in);
      break;
    }
    default: {
      const int c1 = 2 * j + 1, c2 = 2 * j + 2;
      const double out = dbl(f.Q[win[j + 1 + (cmy + 1) * ldc]]);
      const double in = dbl(qc_inner ? restrict_cell<T>(Q, ldq, j, cmy - 1) : QC[j + 1 + cmy * ldc]);
      v = (dbl(DnS[2 * j + my * mx]) * (q(c1 + my * ldq) - q(c1 + (my + 1) * ldq)) +
           dbl(DnS[2 * j + 1 + my * mx]) * (q(c2 + my * ldq) - q(c2 + (my + 1) * ldq))) +
          dbl(cfd[2 * cmy + cmx + j]) * (out - in);
      break;
    }
  }
  return divr(v, hc2, ihc2, pow2);
}

// gather-form corrections of one target coarse cell: contributions in the
// reference's order (fine patch ascending, faces W, E, S, N)
struct CorrCSR {
  const int *cell, *patch, *beg, *item, *jj;   // item = (level-local fine patch << 2) | face
};

template <class T>
__device__ __forceinline__ double add_corrections(double v, const CorrCSR &C, int t, const LevelD &Lf, const LevelD &Lc,
                                                  const FieldsT<T> &f, bool qc_inner) {
  for (int i = C.beg[t]; i < C.beg[t + 1]; ++i) {
    const int it = C.item[i];
    const int fc = it & 3;
    v = v + face_corr(Lf.patches[it >> 2], f, fc, C.jj[i], fc < 2 ? Lc.hx2 : Lc.hy2, fc < 2 ? Lc.ihx2 : Lc.ihy2,
                      Lc.pow2, qc_inner);
  }
  return v;
}

// ---------------------------------------------------------------------------
// FAS coarse load of level k (ebVcycle.m:28-29): one launch with three block
// ranges --
//   [0, nb_ring)            QC ring <- parent Q      (ebTransfer.m:35-55)
//   [nb_ring, +D.nblocks)   F_parent = restrict2(F - op(Q)) + op_c(QC, parent
//                           coefficients) over the footprint (ebCoarseLoad.m:17-32,
//                           ebParentCoeffs.m), the four fine residuals summed in
//                           restrict2 order (1,1), (2,1), (1,2), (2,2)
//   [.., +nb_tgt)           F_target = F_target + corrections (ebCoarseLoad.m:37-45)
// QC ring values are read from the parent's Q through the window table, so
// the three ranges are independent.
// op2d at one cell from preloaded face coefficients (same operation order
// as op_cell)
__device__ __forceinline__ double op_pre(double q, double qe, double qw, double qn, double qs, double dE, double dW,
                                         double dN, double dS, double cc, const LevelD &L) {
  const double feE = dE * (qe - q), feW = dW * (q - qw), fnN = dN * (qn - q), fnS = dS * (q - qs);
  return (divr(-(feE - feW), L.hx2, L.ihx2, L.pow2) - divr(fnN - fnS, L.hy2, L.ihy2, L.pow2)) + cc * q;
}

// the three item kinds of the coarse load (kChain as restrict_item)
template <class T, bool kChain>
__device__ __forceinline__ void load_ring_item(const FieldsT<T> &f, const int *__restrict__ ring,
                                               const int *__restrict__ ring_inst, int ring_off, int n_ring, int t) {
  int src = 0, dst = 0;
  bool on = t < n_ring && (!ring_inst || f.active[__ldg(ring_inst + ring_off + t)]);
  if (on) {
    src = __ldg(ring + 2 * (ring_off + t));
    dst = __ldg(ring + 2 * (ring_off + t) + 1);
  }
  if (kChain) chain_wait();
  if (on) f.QC[dst] = f.Q[src];
}

template <class T, bool kChain>
__device__ __forceinline__ void load_fp_item(const LevelD &L, const LevelD &Lc, const Decomp &D, const FieldsT<T> &f,
                                             int g) {
  if (g >= D.n) {
    if (kChain) chain_wait();
    return;
  }
  const int p = find_patch(D, g / kBlock, g);
  const PatchD &P = L.patches[p];
  if (!f.active[P.inst]) {
    if (kChain) chain_wait();
    return;
  }
  const int mx = P.mx, cmx = mx >> 1, cmy = P.my >> 1, ldq = mx + 2;
  const int s = g - __ldg(D.beg + p);
  const int cj = s / cmx, ci = s - cj * cmx;
  const int q_off = P.q_off, c_off = P.c_off, qc_off = P.qc_off;
  // static operands of the four fine cells (restrict2 order) and of the
  // coarse operator
  const T *DeW = f.DeW + P.dew_off, *DnS = f.DnS + P.dns_off, *CC = f.CC + c_off;
  double dE[4], dW[4], dN[4], dS[4], cf[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int li = 2 * ci + (t & 1), lj = 2 * cj + (t >> 1);
    dE[t] = dbl(__ldg(DeW + (li + 1) + lj * (mx + 1)));
    dW[t] = dbl(__ldg(DeW + li + lj * (mx + 1)));
    dN[t] = dbl(__ldg(DnS + li + (lj + 1) * mx));
    dS[t] = dbl(__ldg(DnS + li + lj * mx));
    cf[t] = dbl(__ldg(CC + li + lj * mx));
  }
  const int ldc = cmx + 2;
  const int *win = f.win + P.win_off;
  const int w = (ci + 1) + (cj + 1) * ldc;
  // ring neighbours of the coarse operator come from the parent's Q
  const int se = (ci == cmx - 1) ? __ldg(win + w + 1) : -1;
  const int sw = (ci == 0) ? __ldg(win + w - 1) : -1;
  const int sn = (cj == cmy - 1) ? __ldg(win + w + ldc) : -1;
  const int ss = (cj == 0) ? __ldg(win + w - ldc) : -1;
  const T *PDeW = f.pcoef + P.pc_off;
  const T *PDnS = PDeW + (cmx + 1) * cmy;
  const T *PCC = PDnS + cmx * (cmy + 1);
  const double pE = dbl(__ldg(PDeW + (ci + 1) + cj * (cmx + 1))), pW = dbl(__ldg(PDeW + ci + cj * (cmx + 1)));
  const double pN = dbl(__ldg(PDnS + ci + (cj + 1) * cmx)), pS = dbl(__ldg(PDnS + ci + cj * cmx));
  const double pC = dbl(__ldg(PCC + s));
  const int dst = __ldg(f.fp + 2 * (P.fp_off + s) + 1);
  if (kChain) chain_wait();
  const T *Qp = f.Q + q_off;
  const T *Fp = f.F + c_off;
  double rf[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int li = 2 * ci + (t & 1), lj = 2 * cj + (t >> 1);
    const int c = (li + 1) + (lj + 1) * ldq;
    rf[t] = dbl(Fp[li + lj * mx]) - op_pre(dbl(Qp[c]), dbl(Qp[c + 1]), dbl(Qp[c - 1]), dbl(Qp[c + ldq]),
                                           dbl(Qp[c - ldq]), dE[t], dW[t], dN[t], dS[t], cf[t], L);
  }
  const double rr = 0.25 * (((rf[0] + rf[1]) + rf[2]) + rf[3]);
  const T *QC = f.QC + qc_off;
  const double q = dbl(QC[w]);
  const double qe = dbl(se >= 0 ? f.Q[se] : QC[w + 1]);
  const double qw = dbl(sw >= 0 ? f.Q[sw] : QC[w - 1]);
  const double qn = dbl(sn >= 0 ? f.Q[sn] : QC[w + ldc]);
  const double qs = dbl(ss >= 0 ? f.Q[ss] : QC[w - ldc]);
  const double lc = op_pre(q, qe, qw, qn, qs, pE, pW, pN, pS, pC, Lc);
  f.F[dst] = T(rr + lc);
}

template <class T, bool kChain>
__device__ __forceinline__ void load_corr_item(const LevelD &L, const LevelD &Lc, const FieldsT<T> &f, const CorrCSR &C,
                                               int n_tgt, int t) {
  const bool on = t < n_tgt && f.active[Lc.patches[C.patch[t]].inst];
  const int cell = on ? C.cell[t] : 0;
  if (kChain) chain_wait();
  if (!on) return;
  // FP64: the target's F before its corrections is FTrue (the value the
  // reference's per-cycle reset F = FTrue leaves there), so the V-cycle does
  // not depend on a reset of F before it; the correction cycle of the mixed
  // form adds to its own right-hand side
  const double base = sizeof(T) == sizeof(double) ? f.FTrue[cell] : dbl(f.F[cell]);
  f.F[cell] = T(add_corrections<T>(base, C, t, L, Lc, f, false));
}

// kT threads per block (kBlock, or 64 on a level whose kBlock grid leaves
// SMs idle: a footprint cell is ~84 FP64 operations, and an SM issues about
// two per clock); the decomposition's per-block patch table is kBlock-based
template <class T, int kT = kBlock>
__global__ void __launch_bounds__(kT) k_load(LevelD L, LevelD Lc, Decomp D, FieldsT<T> f, const int *__restrict__ ring,
                                             const int *__restrict__ ring_inst, int ring_off, int n_ring, CorrCSR C,
                                             int n_tgt) {
  chain_trigger();
  const int nb_ring = (n_ring + kT - 1) / kT;
  const int nb_fp = (D.n + kT - 1) / kT;
  int b = blockIdx.x;
  if (b < nb_ring) {
    load_ring_item<T, true>(f, ring, ring_inst, ring_off, n_ring, b * kT + threadIdx.x);
    return;
  }
  b -= nb_ring;
  if (b < nb_fp) {
    load_fp_item<T, true>(L, Lc, D, f, b * kT + threadIdx.x);
    return;
  }
  b -= nb_fp;
  load_corr_item<T, true>(L, Lc, f, C, n_tgt, b * kT + threadIdx.x);
}

// ---------------------------------------------------------------------------
// prolongBilin (ebKernels.m:105-123) of the parent window: 'correct'
// (ebTransfer.m:57-71) adds P(W - QC) to the interior; mode 0 writes P(W)
// (new-level initial guess, ebAddLevel.m:26-31).  One thread per coarse cell
// writes its four fine cells.
// kT threads per block: kBlock, or 64 on a level whose kBlock grid leaves
// SMs idle (about 37 FP64 operations per coarse cell, two per clock per SM)
// A parent-window operand of the prolongation fused with the parent level's
// closing fill (k_fill_prolong): a code >= 0 is a cell of Q; a code < 0 is
// the ghost cell that ghost item -1 - code fills in the same launch, whose
// value the prolongation forms itself from the item's rule (the rule reads
// interior cells and the level below, which the launch does not write) --
// the value the fill stores, bit for bit.
template <class T>
struct WindowGhosts {
  const int *win;              // window tables, ghost cells coded
  GhostItems G;
  const T *bcg;
  T hx, hy;                    // cell size of the parent level (the ghosts' level)
};

template <class T>
__device__ __forceinline__ T window_value(const T *Q, int code, const WindowGhosts<T> *W) {
  if (W == nullptr || code >= 0) return Q[code];
  const int i = -1 - code;
  const GhostItems &G = W->G;
  const int8_t ty = G.type[i];
  if (ty == G_PHYS_CORNER) {
    const T v1 = eval_rule<T>(G, G.a[i], Q, W->bcg, W->hx, W->hy);
    const T v2 = eval_rule<T>(G, G.b[i], Q, W->bcg, W->hx, W->hy);
    return (v1 + v2) - Q[G.c[i]];
  }
  return eval_rule<T>(G, i, Q, W->bcg, W->hx, W->hy);
}

template <class T, bool kChain>
__device__ __forceinline__ void prolong_item(const LevelD &L, const Decomp &D, const FieldsT<T> &f, int correct,
                                             int g, const WindowGhosts<T> *W = nullptr) {
  if (g >= D.n) {
    if (kChain) chain_wait();
    return;
  }
  const int p = find_patch(D, g / kBlock, g);
  const PatchD &P = L.patches[p];
  if (!f.active[P.inst]) {   // frozen instance, or an instance whose level k is not new
    if (kChain) chain_wait();
    return;
  }
  const int cm = P.mx >> 1;
  const int s = g - __ldg(D.beg + p);
  const int b = s / cm, a = s - b * cm;
  const int ldw = cm + 2;
  const int *win = (W ? W->win : f.win) + P.win_off;
  int src[3][3];
#pragma unroll
  for (int dj = 0; dj < 3; ++dj)
#pragma unroll
    for (int di = 0; di < 3; ++di) src[dj][di] = __ldg(win + (a + di) + (b + dj) * ldw);
  const int qc_off = P.qc_off, q_off = P.q_off, ldq = P.mx + 2;
  if (kChain) chain_wait();
  const T *QC = f.QC + qc_off;
  T E[3][3];
#pragma unroll
  for (int dj = 0; dj < 3; ++dj)
#pragma unroll
    for (int di = 0; di < 3; ++di) {
      const int w = (a + di) + (b + dj) * ldw;
      const T wv = window_value<T>(f.Q, src[dj][di], W);
      E[dj][di] = correct ? wv - QC[w] : wv;
    }
  const T C = E[1][1], Wm = E[1][0], Wp = E[1][2], Sm = E[0][1], Sp = E[2][1];
  const T f11 = (((9 * C + 3 * Wm) + 3 * Sm) + E[0][0]) / 16;
  const T f21 = (((9 * C + 3 * Wp) + 3 * Sm) + E[0][2]) / 16;
  const T f12 = (((9 * C + 3 * Wm) + 3 * Sp) + E[2][0]) / 16;
  const T f22 = (((9 * C + 3 * Wp) + 3 * Sp) + E[2][2]) / 16;
  T *Q = f.Q + q_off;
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

template <class T, int kT = kBlock>
__global__ void __launch_bounds__(kT) k_prolong(LevelD L, Decomp D, FieldsT<T> f, int correct) {
  chain_trigger();
  prolong_item<T, true>(L, D, f, correct, blockIdx.x * kT + threadIdx.x);
}

// The closing ghost fill of level k-1 (the end of its V-cycle) and the
// prolongation-correction of level k that follows it (ebVcycle.m:31-32) in
// one launch: blocks [0, nb_g) fill level k-1, the rest prolong into level
// k, forming any parent-window ghost from its rule (WindowGhosts), so no
// item reads what another item of the launch writes.
template <class T, int kT = kBlock>
__global__ void __launch_bounds__(kT) k_fill_prolong(GhostItems G, int g_off, int g_n, int nb_g, LevelD L, Decomp D,
                                                    FieldsT<T> f, int correct, WindowGhosts<T> W,
                                                    const int *__restrict__ active,
                                                    const int *__restrict__ inst_nlev) {
  chain_trigger();
  if ((int)blockIdx.x < nb_g) {
    const int t = blockIdx.x * kT + threadIdx.x;
    const int i = g_off + t;
    const int inst = (t < g_n && G.inst) ? G.inst[i] : -1;
    const bool skip = t >= g_n || (inst >= 0 && !active[inst]);
    GhostPrep P;
    if (!skip) P = ghost_prep(G, i, G.type[i], G.dst[i]);
    chain_wait();
    if (skip) return;
    ghost_apply<T>(G, i, P, f.Q, f.QC, f.bcg, W.hx, W.hy);
    return;
  }
  prolong_item<T, true>(L, D, f, correct, ((int)blockIdx.x - nb_g) * kT + threadIdx.x, &W);
}

// ---------------------------------------------------------------------------
// Coarsest solve (ebCoarsest.m:79-91): u = Ainv (F + bcRhs), one warp per
// row; lane l sums columns l, l+32, ... in order, then a halving tree.
struct CoarsestD {
  int c_off, q_off, n1, N, inst, pad;
  long long ainv_off, rhs_off;
};

// bcRhs null: a homogeneous problem (the correction cycle of the mixed
// form), whose F is FP32 while the solve itself stays FP64.
// one warp per row, kRows rows per block: one row per block spreads a single
// hierarchy's rows' FP64 work over as many SMs as there are rows; a batch
// keeps eight, since most of its instances' blocks exit at once in its last
// V-cycles
// one row of the coarsest solve, computed by one warp (lane = lane index)
template <class T, bool kChain>
__device__ __forceinline__ void coarsest_row(const double *__restrict__ Ainv, const double *__restrict__ bcRhs,
                                             const CoarsestD &D, const FieldsT<T> &f, int row, int lane) {
  const int N = D.N;
  if (row >= N || !f.active[D.inst]) {
    if (kChain) chain_wait();
    return;
  }
  const double *a = Ainv + D.ainv_off + (size_t)row * N;
  const double *rhs = bcRhs ? bcRhs + D.rhs_off : nullptr;
  constexpr int kPre = 8;   // inverse entries held in registers (N <= 256)
  double av[kPre], bv[kPre];
#pragma unroll
  for (int i = 0; i < kPre; ++i) {
    const int c = lane + 32 * i;
    av[i] = c < N ? __ldg(a + c) : 0.0;
    bv[i] = (c < N && rhs) ? __ldg(rhs + c) : 0.0;
  }
  if (kChain) chain_wait();
  const T *F = f.F + D.c_off;
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < kPre; ++i) {
    const int c = lane + 32 * i;
    if (c < N) s = s + av[i] * (dbl(F[c]) + bv[i]);
  }
  for (int c = lane + 32 * kPre; c < N; c += 32) s = s + a[c] * (dbl(F[c]) + (rhs ? rhs[c] : 0.0));
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    const double o = __shfl_down_sync(0xffffffffu, s, off);
    if (lane < off) s = s + o;
  }
  if (lane == 0) {
    const int i = row % D.n1, j = row / D.n1;
    f.Q[D.q_off + (i + 1) + (j + 1) * (D.n1 + 2)] = T(s);
  }
}

template <class T, int kRows = 1>
__global__ void __launch_bounds__(32 * kRows) k_coarsest(const double *__restrict__ Ainv,
                                                         const double *__restrict__ bcRhs,
                                                         const CoarsestD *__restrict__ cd, FieldsT<T> f) {
  chain_trigger();
  const CoarsestD D = cd[blockIdx.y];
  coarsest_row<T, true>(Ainv, bcRhs, D, f, blockIdx.x * kRows + (int)(threadIdx.x >> 5), threadIdx.x & 31);
}

// ---------------------------------------------------------------------------
// Composite residual (ebCompResidual.m:15-85) of every level >= root, for one
// hierarchy or every instance of a batch, in one launch.  The work is a list
// of warp tasks, each covering up to 32 * kResLane items of ONE patch (or of
// one instance's correction targets), so every warp belongs to one instance:
//   kind 0  r = FTrue - op(Q) on visible cells of a patch in the norms,
//           correction targets excluded while the corrections are on
//   kind 1  r at correction targets of a level, corrections added in order,
//           the coarse values taken as the refreshed QC holds them
//   kind 2  QC ring refresh of a patch (ebCompResidual.m:25)
//   kind 3  QC interior refresh of a patch (ebCompResidual.m:32-38)
// A residual warp reduces its values (fixed shuffle tree) into one slot;
// k_residual_final reduces each instance's slots.  Max-norms are order-free,
// so linf and rel do not depend on the task layout.
struct ResAcc {
  double out[5];        // linf, l2, fnorm, rel, ncell
};

struct ResTask {
  int kind, level, a, b, n, slot, inst, pad;   // a: patch / CSR level / ring start; b: first item
};

struct LevelX {
  LevelD L;
  CorrCSR C;            // corrections contributed by this (fine) level
  int ct_n, pad;
};

// max of non-negative doubles on the integer pipe (their bit patterns order
// like the values; the FP64 pipe of GB300 is the scarce one).  A NaN loses,
// as in fmax and the reference's max: its pattern ranks below zero here.
__device__ __forceinline__ double pmax(double a, double b) {
  constexpr long long kInf = 0x7FF0000000000000LL;
  long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  x = x > kInf ? -1 : x;
  y = y > kInf ? -1 : y;
  const long long m = x > y ? x : y;
  return __longlong_as_double(m < 0 ? 0 : m);
}

// items per lane of a residual warp task (a task covers up to 32 * kResLane
// items of one patch or one instance's targets)
constexpr int kResLane = 4;

// kT threads per block (kBlock, or 64 where the kBlock grid would leave
// SMs with unequal shares of the FP64 work)
template <int kT = kBlock>
__global__ void __launch_bounds__(kT) k_residual(const LevelX *__restrict__ X, const PatchD *__restrict__ patches,
                                                 const ResTask *__restrict__ tasks, int ntask, Fields f,
                                                 const int *__restrict__ ring, double *slots, int nslots,
                                                 int mass_corr, float *__restrict__ rout) {
  chain_trigger();
  const int w = blockIdx.x * (kT / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  // a frozen instance's residual is neither reported nor needed (its QC
  // refresh would rewrite the same values), so its warps only wait
  if (w >= ntask || !f.active[tasks[w].inst]) {
    chain_wait();
    return;
  }
  const ResTask T = tasks[w];
  chain_wait();
  if (T.kind >= 2) {
    if (!mass_corr) return;
    if (T.kind == 2) {
      for (int e = lane; e < T.n; e += 32) {
        const int i = T.a + e;
        f.QC[__ldg(ring + 2 * i + 1)] = f.Q[__ldg(ring + 2 * i)];
      }
      return;
    }
    const PatchD &P = patches[T.a];
    const int cmx = P.mx >> 1;
    for (int e = lane; e < T.n; e += 32) {
      const int s = T.b + e;
      const int cj = s / cmx, ci = s - cj * cmx;
      f.QC[P.qc_off + (ci + 1) + (cj + 1) * (cmx + 2)] = restrict_cell(f.Q + P.q_off, P.mx + 2, ci, cj);
    }
    return;
  }
  double li = 0, sq = 0, fn = 0;
  const LevelX &Xk = X[T.level];
  if (T.kind == 0) {
    const PatchD &P = patches[T.a];
    const int mx = P.mx, ldq = mx + 2;
    const double *DeW = f.DeW + P.dew_off, *DnS = f.DnS + P.dns_off, *Qp = f.Q + P.q_off;
#pragma unroll
    for (int u = 0; u < kResLane; ++u) {
      const int e = lane + 32 * u;
      if (e >= T.n) break;
      const int s = T.b + e;
      const int lj = s / mx, lx = s - lj * mx;
      const int cc = P.c_off + s;
      const uint8_t fl = __ldg(f.flags + cc);
      if ((fl & 1) || (mass_corr && (fl & 2))) continue;
      const double ft = __ldg(f.FTrue + cc);
      const int c = (lx + 1) + (lj + 1) * ldq;
      const double r = ft - op_pre(Qp[c], Qp[c + 1], Qp[c - 1], Qp[c + ldq], Qp[c - ldq],
                                   __ldg(DeW + (lx + 1) + lj * (mx + 1)), __ldg(DeW + lx + lj * (mx + 1)),
                                   __ldg(DnS + lx + (lj + 1) * mx), __ldg(DnS + lx + lj * mx), __ldg(f.CC + cc), Xk.L);
      li = pmax(li, fabs(r));
      sq = sq + r * r;
      fn = pmax(fn, fabs(ft));
      if (rout) rout[cc] = (float)r;
    }
  } else if (mass_corr) {   // kind 1: targets of this level, corrections from the level above
    const LevelX &Xf = X[T.level + 1];
    for (int u = 0; u < kResLane; ++u) {
      const int e = lane + 32 * u;
      if (e >= T.n) break;
      const int g = T.b + e;
      const int cell = Xf.C.cell[g];
      const PatchD &Pc = Xk.L.patches[Xf.C.patch[g]];
      const int s = cell - Pc.c_off;
      const int lj = s / Pc.mx, lx = s - lj * Pc.mx;
      const double ft = f.FTrue[cell];
      double r = ft - op_cell_r(f.Q + Pc.q_off, Pc.mx + 2, f.DeW + Pc.dew_off, f.DnS + Pc.dns_off, f.CC[cell], Pc.mx,
                                lx, lj, Xk.L);
      r = add_corrections(r, Xf.C, g, Xf.L, Xk.L, f, true);
      if (rout) rout[cell] = (float)r;
      if (!(f.flags[cell] & 1)) {
        li = pmax(li, fabs(r));
        sq = sq + r * r;
        fn = pmax(fn, fabs(ft));
      }
    }
  }
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    li = pmax(li, __shfl_down_sync(0xffffffffu, li, off));
    fn = pmax(fn, __shfl_down_sync(0xffffffffu, fn, off));
    sq = sq + __shfl_down_sync(0xffffffffu, sq, off);
  }
  if (lane == 0) {
    slots[T.slot] = li;
    slots[nslots + T.slot] = sq;
    slots[2 * nslots + T.slot] = fn;
  }
}

// per instance: the slot ranges of its residual tasks, level by level
struct InstRes {
  int range0, range1;   // into the (slot0, slot1, level area) range table
  int max_vcycles, pad;
  double rel_tol, ncell;
};

struct SlotRange {
  int s0, s1;
  double area;
};

// finish the residual of every instance (one block per instance): max-norms
// over its slots, L2 per level from that level's slots in a fixed tree order
// weighted by the cell area, rel = linf / max(fnorm, realmin).  mode 0 is
// the residual before the first V-cycle; mode 1 follows a V-cycle of the
// instances active during it; mode 2 only reports (an eager call).  The history and the stop test follow
// ebSolveCycles.m:17-46: an instance stays active while it < MaxVCycles and
// rel > RelTol.
constexpr int kFinal = 512;
constexpr int kFinalGroup = 8;   // levels whose L2 trees share barrier steps
__global__ void __launch_bounds__(kFinal) k_residual_final(const InstRes *__restrict__ ir,
                                                          const SlotRange *__restrict__ ranges, const double *slots,
                                                          int nslots, ResAcc *acc, int *active, int *iters,
                                                          double *hist, int hist_stride, int mode,
                                                          const int *__restrict__ crange, int nlev, uint8_t *cact) {
  chain_in();
  const int inst = blockIdx.x;
  const InstRes R = ir[inst];
  __shared__ int s_write;
  const int t = threadIdx.x;
  // one pass over the slots: the max-norms (order-free) and, per level
  // (range), a fixed-order tree over the threads' partial sums -- four
  // strided partial sums per thread, then their sum; the levels of a group
  // are reduced in the same barrier steps (each level's pairings unchanged)
  // and summed in level order with their areas
  double li = 0, fn = 0;
  __shared__ double s_p[kFinalGroup][kFinal];
  __shared__ double s_a[kFinal / 32 + 1], s_b[kFinal / 32 + 1];
  double l2sq = 0;
  for (int r0 = R.range0; r0 < R.range1; r0 += kFinalGroup) {
    const int nr = min(kFinalGroup, R.range1 - r0);
    for (int q = 0; q < nr; ++q) {
      const int s0 = ranges[r0 + q].s0, s1 = ranges[r0 + q].s1;
      double p0 = 0, p1 = 0, p2 = 0, p3 = 0;
      int i = s0 + t;
      for (; i + 3 * kFinal < s1; i += 4 * kFinal) {
        const double a0 = slots[i], a1 = slots[i + kFinal], a2 = slots[i + 2 * kFinal], a3 = slots[i + 3 * kFinal];
        const double b0 = slots[2 * nslots + i], b1 = slots[2 * nslots + i + kFinal];
        const double b2 = slots[2 * nslots + i + 2 * kFinal], b3 = slots[2 * nslots + i + 3 * kFinal];
        p0 = p0 + slots[nslots + i];
        p1 = p1 + slots[nslots + i + kFinal];
        p2 = p2 + slots[nslots + i + 2 * kFinal];
        p3 = p3 + slots[nslots + i + 3 * kFinal];
        li = pmax(li, pmax(pmax(a0, a1), pmax(a2, a3)));
        fn = pmax(fn, pmax(pmax(b0, b1), pmax(b2, b3)));
      }
      for (; i < s1; i += kFinal) {
        p0 = p0 + slots[nslots + i];
        li = pmax(li, slots[i]);
        fn = pmax(fn, slots[2 * nslots + i]);
      }
      s_p[q][t] = (p0 + p1) + (p2 + p3);
    }
    __syncthreads();
    for (int off = kFinal / 2; off >= 1; off >>= 1) {
      if (t < off)
        for (int q = 0; q < nr; ++q) s_p[q][t] = s_p[q][t] + s_p[q][t + off];
      __syncthreads();
    }
    for (int q = 0; q < nr; ++q) l2sq = l2sq + s_p[q][0] * ranges[r0 + q].area;
    __syncthreads();
  }
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    li = pmax(li, __shfl_xor_sync(0xffffffffu, li, off));
    fn = pmax(fn, __shfl_xor_sync(0xffffffffu, fn, off));
  }
  if ((t & 31) == 0) {
    s_a[t >> 5] = li;
    s_b[t >> 5] = fn;
  }
  __syncthreads();
  if (t < 32) {
    li = t < kFinal / 32 ? s_a[t] : 0.0;
    fn = t < kFinal / 32 ? s_b[t] : 0.0;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
      li = pmax(li, __shfl_xor_sync(0xffffffffu, li, off));
      fn = pmax(fn, __shfl_xor_sync(0xffffffffu, fn, off));
    }
    if (t == 0) {
      s_a[kFinal / 32] = li;
      s_b[kFinal / 32] = fn;
    }
  }
  __syncthreads();
  const double linf = s_a[kFinal / 32];
  double fnorm = s_b[kFinal / 32];
  if (t == 0) {
    int wr = -1;
    fnorm = fnorm > 2.2250738585072014e-308 ? fnorm : 2.2250738585072014e-308;
    const double rel = linf / fnorm;
    ResAcc &A = acc[inst];
    if (mode == 2 || mode == 0 || active[inst]) {
      A.out[0] = linf;
      A.out[1] = sqrt(l2sq);
      A.out[2] = fnorm;
      A.out[3] = rel;
      A.out[4] = R.ncell;
    }
    if (mode != 2 && (mode == 0 || active[inst])) {
      int it = iters[inst];
      if (mode == 0) it = 0;
      else it = it + 1;
      iters[inst] = it;
      if (it < hist_stride) hist[(size_t)inst * hist_stride + it] = linf;
      const int a = (it < R.max_vcycles && rel > R.rel_tol) ? 1 : 0;
      active[inst] = a;
      if (mode == 0 || !a) wr = a;     // every instance at the start; later only when it freezes
    }
    s_write = wr;
  }
  // the smoother's per-chunk copy of the flag, over the instance's chunk
  // range of every level (crange: [inst][level] begin, end)
  if (cact) {
    __syncthreads();
    const int wr = s_write;
    if (wr >= 0)
      for (int k = 0; k < nlev; ++k) {
        const int b = crange[2 * (inst * nlev + k)], e = crange[2 * (inst * nlev + k) + 1];
        for (int c = b + t; c < e; c += kFinal) cact[c] = (uint8_t)wr;
      }
  }
}

// ---------------------------------------------------------------------------
// FP64 issue-rate probe (bsam_fp64_rate): eight independent x = x*a + b
// chains per thread, each a separate multiply and add (the library is built
// without contraction), so 16 FP64 operations per iteration.
constexpr int kFp64RateOps = 16;
__global__ void __launch_bounds__(kBlock) k_fp64_rate(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) x[u] = 1.0 + 1e-3 * u + 1e-9 * threadIdx.x;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 8; ++u) x[u] = x[u] * a + b;
  }
  double s = 0;
#pragma unroll
  for (int u = 0; u < 8; ++u) s = s + x[u];
  out[blockIdx.x * kBlock + threadIdx.x] = s;
}

// ---------------------------------------------------------------------------
// Condition of the solve loop's device-side WHILE node: 1 while any instance
// still iterates (ebSolveCycles.m:22, per instance).  One block; a single
// thread sets the condition.
__global__ void __launch_bounds__(kBlock) k_any_active(const int *__restrict__ active, int ninst,
                                                       cudaGraphConditionalHandle cond,
                                                       cudaGraphConditionalHandle cond2, int use2) {
  chain_in();
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < ninst; i += kBlock)
    if (active[i]) any = 1;   // benign: every writer stores 1
  __syncthreads();
  if (threadIdx.x == 0) {
    cudaGraphSetConditional(cond, any ? 1u : 0u);
    if (use2) cudaGraphSetConditional(cond2, any ? 1u : 0u);
  }
}

// ---------------------------------------------------------------------------
// Force reset F = FTrue (ebSolveCycles.m:30-34) of the active instances of a
// batch, one thread per cell over every patch of every level (a single
// hierarchy copies the whole array instead).
__global__ void __launch_bounds__(kBlock) k_freset(Decomp D, const PatchD *__restrict__ patches, Fields f) {
  chain_trigger();
  const int g = blockIdx.x * kBlock + threadIdx.x;
  if (g >= D.n) {
    chain_wait();
    return;
  }
  const int p = find_patch(D, blockIdx.x, g);
  const PatchD &P = patches[p];
  if (!f.active[P.inst]) {
    chain_wait();
    return;
  }
  const int cc = P.c_off + (g - __ldg(D.beg + p));
  const double v = __ldg(f.FTrue + cc);
  chain_wait();
  f.F[cc] = v;
}

// ---------------------------------------------------------------------------
// Defect correction of the mixed form: Q += E (FP64 += FP32) on the interior
// cells of every patch of the active instances.
__global__ void __launch_bounds__(kBlock) k_update(Decomp D, const PatchD *__restrict__ patches, double *Q,
                                                   const float *__restrict__ E, const int *__restrict__ active) {
  chain_trigger();
  const int g = blockIdx.x * kBlock + threadIdx.x;
  if (g >= D.n) {
    chain_wait();
    return;
  }
  const int p = find_patch(D, blockIdx.x, g);
  const PatchD &P = patches[p];
  if (!active[P.inst]) {
    chain_wait();
    return;
  }
  const int s = g - __ldg(D.beg + p);
  const int lj = s / P.mx, lx = s - lj * P.mx;
  const int qi = P.q_off + (lx + 1) + (lj + 1) * (P.mx + 2);
  chain_wait();
  Q[qi] = Q[qi] + (double)E[qi];
}

// Mixed form: Q += E of the correction cycle (k_update) and the restriction
// of the finest level k (k_restrict) in one launch, where the consistency
// step starts with that plain restriction: blocks [0, nb_r) restrict level
// k, each item adding E to its four fine cells first (k_update's sum) and
// restricting the sums (restrict_cell's order); the other blocks add E to
// the cells of the levels below k that no finer level covers.  A covered
// cell is rewritten by a restriction before anything reads it, and the ones
// this launch's restriction writes must not be touched here, so skipping
// them gives the values of k_update then k_restrict.
template <int kT = kBlock>
__global__ void __launch_bounds__(kT) k_restrict_update(LevelD L, Decomp D, Fields f, const float *__restrict__ E,
                                                       int nb_r, Decomp Du, const PatchD *__restrict__ patches) {
  chain_trigger();
  if ((int)blockIdx.x < nb_r) {
    const int g = blockIdx.x * kT + threadIdx.x;
    if (g >= D.n) {
      chain_wait();
      return;
    }
    const int p = find_patch(D, g / kBlock, g);
    const PatchD &P = L.patches[p];
    if (!f.active[P.inst]) {
      chain_wait();
      return;
    }
    const int cmx = P.mx >> 1, ldq = P.mx + 2;
    const int s = g - __ldg(D.beg + p);
    const int cj = s / cmx, ci = s - cj * cmx;
    const int dst = __ldg(f.fp + 2 * (P.fp_off + s));
    chain_wait();
    double *Q = f.Q + P.q_off;
    const float *e = E + P.q_off;
    const int c = (2 * ci + 1) + (2 * cj + 1) * ldq;
    const double q0 = Q[c] + (double)e[c], q1 = Q[c + 1] + (double)e[c + 1];
    const double q2 = Q[c + ldq] + (double)e[c + ldq], q3 = Q[c + ldq + 1] + (double)e[c + ldq + 1];
    Q[c] = q0;
    Q[c + 1] = q1;
    Q[c + ldq] = q2;
    Q[c + ldq + 1] = q3;
    const double R = 0.25 * (((q0 + q1) + q2) + q3);
    f.QC[P.qc_off + (ci + 1) + (cj + 1) * (cmx + 2)] = R;
    f.Q[dst] = R;
    return;
  }
  const int g = ((int)blockIdx.x - nb_r) * kT + threadIdx.x;
  if (g >= Du.n) {
    chain_wait();
    return;
  }
  const int p = find_patch(Du, g / kBlock, g);
  const PatchD &P = patches[p];
  const int s = g - __ldg(Du.beg + p);
  if (!f.active[P.inst] || (__ldg(f.flags + P.c_off + s) & 1)) {
    chain_wait();
    return;
  }
  const int lj = s / P.mx, lx = s - lj * P.mx;
  const int qi = P.q_off + (lx + 1) + (lj + 1) * (P.mx + 2);
  chain_wait();
  f.Q[qi] = f.Q[qi] + (double)E[qi];
}

// Parabolic driver on the device.  k_history: Uoo = Uo, Uo = interior of Q
// (ebpSolve.m:52-56); with rotate 0 only Uo = interior of Q (the new
// hierarchy's Uo after a regrid, ebpRegrid.m:49).  k_prhs: FTrue of the step
// on the cells of levels at or above the root (ebpRhs.m:25-47): BE f + Uo/Dt,
// BDF2 f + (2 Uo - 0.5 Uoo)/Dt, in that operation order; f null is f = 0.
__global__ void __launch_bounds__(kBlock) k_history(Decomp D, const PatchD *__restrict__ patches, const double *Q,
                                                    double *Uo, double *Uoo, int rotate) {
  chain_in();
  const int g = blockIdx.x * kBlock + threadIdx.x;
  if (g >= D.n) return;
  const int p = find_patch(D, blockIdx.x, g);
  const PatchD &P = patches[p];
  const int s = g - __ldg(D.beg + p);
  const int lj = s / P.mx, lx = s - lj * P.mx;
  const int cc = P.c_off + s;
  if (rotate) Uoo[cc] = Uo[cc];
  Uo[cc] = Q[P.q_off + (lx + 1) + (lj + 1) * (P.mx + 2)];
}

// The BDF2 history Uoo of one level of a regridded hierarchy
// (ebpRegrid.m:62-137, transferLevel): where a patch of the old hierarchy
// on the same level covers the cell (src_old >= 0, an index into the old
// hierarchy's cells) its old value is copied; elsewhere the value is the
// conservative-linear prolongation of the new parent level's (already
// transferred) history over the patch footprint (conslinInterior +
// parentFootprint: central slopes inside the footprint, one-sided at its
// edges, none along a footprint one coarse cell wide), in the reference's
// operation order.  The footprint's parent cells come from the footprint
// table (second entry per coarse cell); the root level copies every cell.
__global__ void __launch_bounds__(kBlock) k_uoo_transfer(LevelD L, Decomp D, const int *__restrict__ fp,
                                                         const int *__restrict__ src_old,
                                                         const double *__restrict__ uoo_old, double *uoo) {
  chain_in();
  const int g = blockIdx.x * kBlock + threadIdx.x;
  if (g >= D.n) return;
  const int p = find_patch(D, blockIdx.x, g);
  const PatchD &P = L.patches[p];
  const int s = g - __ldg(D.beg + p);
  const int c = P.c_off + s;
  const int so = src_old[c];
  if (so >= 0) {
    uoo[c] = uoo_old[so];
    return;
  }
  const int mx = P.mx, lj = s / mx, li = s - lj * mx;
  const int cmx = mx >> 1, cmy = P.my >> 1, ci = li >> 1, cj = lj >> 1;
  const int *pc = fp + 2 * P.fp_off + 1;      // parent cell of footprint cell t at pc[2 t]
  auto at = [&](int a, int b) { return uoo[pc[2 * (a + b * cmx)]]; };
  const double v = at(ci, cj);
  double sx = 0, sy = 0;
  if (cmx > 1) sx = ci == 0 ? at(1, cj) - v : (ci == cmx - 1 ? v - at(ci - 1, cj) : (at(ci + 1, cj) - at(ci - 1, cj)) / 2);
  if (cmy > 1) sy = cj == 0 ? at(ci, 1) - v : (cj == cmy - 1 ? v - at(ci, cj - 1) : (at(ci, cj + 1) - at(ci, cj - 1)) / 2);
  const double a = (li & 1) ? v + sx / 4 : v - sx / 4;
  uoo[c] = (lj & 1) ? a + sy / 4 : a - sy / 4;
}

__global__ void __launch_bounds__(kBlock) k_prhs(Decomp D, const PatchD *__restrict__ patches, double *FTrue,
                                                 const double *__restrict__ fsrc, const double *__restrict__ Uo,
                                                 const double *__restrict__ Uoo, double dt, int bdf2) {
  chain_in();
  const int g = blockIdx.x * kBlock + threadIdx.x;
  if (g >= D.n) return;
  const int p = find_patch(D, blockIdx.x, g);
  const PatchD &P = patches[p];
  if (!(P.pflags & 1)) return;               // below the root
  const int cc = P.c_off + (g - __ldg(D.beg + p));
  const double f = fsrc ? fsrc[cc] : 0.0;
  FTrue[cc] = bdf2 ? f + (2 * Uo[cc] - 0.5 * Uoo[cc]) / dt : f + Uo[cc] / dt;
}

// ---------------------------------------------------------------------------
// Tagging indicators on the device (ebTagCluster.m:50-59 'ulap',
// ebRte.m:14-41 'rte'), on the finest level's index space (n0 x n1, stored
// i-major: index i * n1 + j).  Only the final mask goes to the host, where
// Berger-Rigoutsos clustering runs.  The arithmetic is the host
// restatement's, in its order, so the masks are identical.
__global__ void __launch_bounds__(kBlock) k_tag_ulap(LevelD L, Decomp D, const double *__restrict__ Q, double thr,
                                                     uint8_t *T, uint8_t *cover, int n1) {
  const int g = blockIdx.x * kBlock + threadIdx.x;
  if (g >= D.n) return;
  const int p = find_patch(D, blockIdx.x, g);
  const PatchD &P = L.patches[p];
  const int s = g - __ldg(D.beg + p);
  const int lj = s / P.mx, li = s - lj * P.mx;
  const int ldq = P.mx + 2;
  const double *q = Q + P.q_off + (li + 1) + (lj + 1) * ldq;
  const double sdx = (q[1] - 2 * q[0]) + q[-1];
  const double sdy = (q[ldq] - 2 * q[0]) + q[-ldq];
  const double v = sqrt(sdx * sdx + sdy * sdy);
  const size_t o = (size_t)(P.ilo - 1 + li) * n1 + (P.jlo - 1 + lj);
  cover[o] = 1;
  if (v > thr) T[o] = 1;
}

// relative truncation error: |op_2h(R u) - R(op_h u)| per coarse cell,
// spread to its four fine cells
__global__ void __launch_bounds__(kBlock) k_tag_rte(LevelD L, Decomp D, Fields f, double thr, uint8_t *T,
                                                    uint8_t *cover, int n1) {
  const int g = blockIdx.x * kBlock + threadIdx.x;
  if (g >= D.n) return;
  const int p = find_patch(D, blockIdx.x, g);
  const PatchD &P = L.patches[p];
  const int mx = P.mx, my = P.my, cmx = mx >> 1, cmy = my >> 1, ldq = mx + 2;
  const int s = g - __ldg(D.beg + p);
  const int cj = s / cmx, ci = s - cj * cmx;
  const double *Q = f.Q + P.q_off, *DeW = f.DeW + P.dew_off, *DnS = f.DnS + P.dns_off, *CC = f.CC + P.c_off;
  double Lf[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int li = 2 * ci + (t & 1), lj = 2 * cj + (t >> 1);
    Lf[t] = op_cell_r(Q, ldq, DeW, DnS, CC[li + lj * mx], mx, li, lj, L);
  }
  const double RL = 0.25 * (((Lf[0] + Lf[1]) + Lf[2]) + Lf[3]);
  // the restricted solution and its ghost frame (pair averages of fine ghosts)
  const double rc = restrict_cell(Q, ldq, ci, cj);
  const double re = ci + 1 < cmx ? restrict_cell(Q, ldq, ci + 1, cj)
                                 : 0.5 * (Q[(mx + 1) + (2 * cj + 1) * ldq] + Q[(mx + 1) + (2 * cj + 2) * ldq]);
  const double rw = ci > 0 ? restrict_cell(Q, ldq, ci - 1, cj) : 0.5 * (Q[(2 * cj + 1) * ldq] + Q[(2 * cj + 2) * ldq]);
  const double rn = cj + 1 < cmy ? restrict_cell(Q, ldq, ci, cj + 1)
                                 : 0.5 * (Q[(2 * ci + 1) + (my + 1) * ldq] + Q[(2 * ci + 2) + (my + 1) * ldq]);
  const double rs = cj > 0 ? restrict_cell(Q, ldq, ci, cj - 1) : 0.5 * (Q[2 * ci + 1] + Q[2 * ci + 2]);
  // averaged coarse coefficients
  const double cE = 0.5 * (DeW[(2 * ci + 2) + (2 * cj) * (mx + 1)] + DeW[(2 * ci + 2) + (2 * cj + 1) * (mx + 1)]);
  const double cW = 0.5 * (DeW[(2 * ci) + (2 * cj) * (mx + 1)] + DeW[(2 * ci) + (2 * cj + 1) * (mx + 1)]);
  const double cN = 0.5 * (DnS[(2 * ci) + (2 * cj + 2) * mx] + DnS[(2 * ci + 1) + (2 * cj + 2) * mx]);
  const double cS = 0.5 * (DnS[(2 * ci) + (2 * cj) * mx] + DnS[(2 * ci + 1) + (2 * cj) * mx]);
  const double cC = 0.25 * (((CC[2 * ci + 2 * cj * mx] + CC[2 * ci + 1 + 2 * cj * mx]) + CC[2 * ci + (2 * cj + 1) * mx]) +
                            CC[2 * ci + 1 + (2 * cj + 1) * mx]);
  const double H2x = (2 * L.hx) * (2 * L.hx), H2y = (2 * L.hy) * (2 * L.hy);
  const double feE = cE * (re - rc), feW = cW * (rc - rw), fnN = cN * (rn - rc), fnS = cS * (rc - rs);
  const double tau = ((-(feE - feW)) / H2x - (fnN - fnS) / H2y + cC * rc) - RL;
  const bool tag = fabs(tau) > thr;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int li = 2 * ci + (t & 1), lj = 2 * cj + (t >> 1);
    const size_t o = (size_t)(P.ilo - 1 + li) * n1 + (P.jlo - 1 + lj);
    cover[o] = 1;
    if (tag) T[o] = 1;
  }
}

// dilate by b cells (outside the index space counts as untagged), then keep
// what the 8-eroded patch cover allows (outside counts as covered)
__global__ void __launch_bounds__(kBlock) k_tag_buffer(const uint8_t *__restrict__ T, const uint8_t *__restrict__ cover,
                                                       uint8_t *out, int n0, int n1, int b) {
  const long long g = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (g >= (long long)n0 * n1) return;
  const int i = (int)(g / n1), j = (int)(g - (long long)i * n1);
  bool t = false;
  for (int dx = -b; dx <= b && !t; ++dx)
    for (int dy = -b; dy <= b; ++dy) {
      const int ii = i + dx, jj = j + dy;
      if (ii >= 0 && ii < n0 && jj >= 0 && jj < n1 && T[(size_t)ii * n1 + jj]) {
        t = true;
        break;
      }
    }
  bool a = true;
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy) {
      const int ii = i + dx, jj = j + dy;
      if (ii >= 0 && ii < n0 && jj >= 0 && jj < n1 && !cover[(size_t)ii * n1 + jj]) a = false;
    }
  out[g] = (t && a) ? 1 : 0;
}

// FP32 copy of an FP64 array (coefficient copies of the mixed form)
__global__ void __launch_bounds__(kBlock) k_to_f32(const double *__restrict__ a, float *__restrict__ b, long long n) {
  chain_in();
  for (long long i = blockIdx.x * (long long)kBlock + threadIdx.x; i < n; i += (long long)gridDim.x * kBlock)
    b[i] = (float)a[i];
}

// ---------------------------------------------------------------------------
// Composite sums over visible cells (ebCompositeMean.m, ebMassCheck.m lhs):
// per-block partials of sum(u), sum(C u - FTrue), sum(|FTrue|)
__global__ void __launch_bounds__(kBlock) k_sums(LevelD L, Decomp D, Fields f, double *partials) {
  chain_in();
  const int g = blockIdx.x * kBlock + threadIdx.x;
  double su = 0, sm = 0, sa = 0, nv = 0;
  if (g < D.n) {
    const int p = find_patch(D, blockIdx.x, g);
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
