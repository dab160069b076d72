// bsam_dev.cu -- C-ABI, hierarchy residency and launch sequencing of the
// GB300 solve path (include/bsam_dev.h).
//
// Upload turns the reference-structured flat tables into an execution plan:
//   * per level, work decompositions over colour cells, cells and coarse
//     cells (256-item blocks, several small patches per block);
//   * per level, a ghost program: one final rule per ghost cell resolved from
//     the three ordered stages of ebFillGhosts, plus the QC ring refresh;
//   * per fine level, the flux corrections in gather form (CSR over target
//     coarse cells, contributions in the reference's order);
//   * residual reduction slots and the coarsest inverse.
// One V-cycle + fill-down + residual is a fixed launch sequence, captured
// once into a CUDA graph per hierarchy and replayed each cycle.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <unordered_map>
#include <mutex>
#include <string>
#include <vector>

#include "bsam_dev.h"
#include "internal.h"
#include "kernels.cuh"

using namespace bsam;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(e == cudaErrorMemoryAllocation ? BSAM_ERR_NOMEM : BSAM_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(x)                                     \
  do {                                            \
    cudaError_t e_ = (x);                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, #x); \
  } while (0)

// flat.py column layouts
enum { LD_N0, LD_N1, LD_P0, LD_P1, LD_CELL0, LD_CELL1, LD_Q0, LD_Q1, LDN };
enum {
  PD_LEVEL, PD_ILO, PD_IHI, PD_JLO, PD_JHI, PD_MX, PD_MY, PD_PAR0,
  PD_BCW, PD_BCE, PD_BCS, PD_BCN, PD_FIW, PD_FIE, PD_FIS, PD_FIN,
  PD_CCSW, PD_CCSE, PD_CCNW, PD_CCNE,
  PD_QOFF, PD_COFF, PD_DEWOFF, PD_DNSOFF, PD_QCOFF, PD_BCGOFF, PD_CFDOFF, PD_PCOFF,
  PD_SAME0, PD_SAME1, PD_RING0, PD_RING1, PD_WIN0, PD_FP0, PD_CORR0, PD_PARENT, PDN
};

// the stream of the hierarchy the calling thread is working on (set by
// set_device): device buffers are allocated and freed in its order from the
// device's memory pool, so setting up or tearing down one hierarchy never
// waits for the work other hierarchies have in flight on other streams (a
// plain cudaFree synchronises the whole device)
thread_local cudaStream_t g_stream = nullptr;

template <class T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;
  int alloc(size_t count) {
    n = count;
    if (count == 0) return BSAM_OK;
    s = g_stream;
    CK(cudaMallocAsync((void **)&p, sizeof(T) * count, s));
    return BSAM_OK;
  }
  int upload(const T *h, size_t count, cudaStream_t s) {
    int rc = alloc(count);
    if (rc) return rc;
    if (count) CK(cudaMemcpyAsync(p, h, sizeof(T) * count, cudaMemcpyHostToDevice, s));
    return BSAM_OK;
  }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    n = 0;
  }
};

bool is_pow2(double x) {
  int e;
  return x > 0 && std::frexp(x, &e) == 0.5;
}

struct DecompH {
  int beg_off = 0, blk_off = 0, n = 0, nblocks = 0;
};

struct LevelPlan {
  int k = 0, p0 = 0, p1 = 0;  // global patch range
  double hx = 0, hy = 0;
  bool pow2 = false;
  DecompH col, cell, coarse;
  int g1_off = 0, g1_n = 0;
  int rc_off = 0, rc_n = 0;        // relax chunk records
  int ring_off = 0, ring_n = 0;
  // corrections contributed by this (fine) level, targets in level k-1
  int ct_off = 0, ct_n = 0;
  int64_t ncells = 0;
  // may this level's own closing fill join the launch of its restriction
  // into the parent (k_restrict_fill): after the pre-smoothing (ring items
  // left out), and with its ring items before the fill-down (set at upload)
  bool fuse_pre = false, fuse_top = false;
  // does a ghost rule of this level read a ghost cell of the parent level
  bool reads_pg = true;
  int64_t q_lo = 0, q_hi = 0;      // the level's patches' range of Q (ghosts included)
  bool range_own = false;          // no other level's patch lies inside [q_lo, q_hi)
  int dsm_shift[2] = {-1, -1};     // k_relax_dsm slice size 2^shift per precision (-1: not a candidate)
};

}  // namespace

// error reporting shared with the other translation units of the library
int bsam_internal_set_error(int code, const std::string &msg) { return fail(code, msg); }


struct bsam_hier_s {
  bsam_ctx ctx = nullptr;
  cudaStream_t stream = nullptr;
  int nlev = 0, root = 0, npatch = 0;
  bsam_solve_opts opts{};
  std::vector<int32_t> hpatches;  // host copy of the descriptor table
  std::vector<int32_t> hlevels;
  std::vector<double> hs;
  std::vector<LevelPlan> lev;     // index 1..nlev
  int64_t n_q = 0, n_cells = 0, n_qc = 0;
  int ninst = 1;                   // instances (a single hierarchy is one instance)
  std::vector<int> inst_root;
  std::vector<int64_t> inst_visible;
  int64_t ncoarse_total = 0;
  int ncoarse_patches = 0, coarse_max_rows = 0;
  // device arrays
  DBuf<double> Q, F, FTrue, QC, CC, ID, DeW, DnS, bcg, cfd, pcoef, Ainv, bcRhs, slots, partials, hist;
  DBuf<uint8_t> flags;
  DBuf<int> win, fp, ring, ints, ct_cell, ct_patch, ct_beg, ct_item, ct_j, active, iters, ones;
  DBuf<int> g_inst, ring_inst;     // instance per ghost item / ring entry (batches only)
  DBuf<int> inst_nlev;             // per instance: its finest level
  // mixed form: FP32 correction, its right-hand side and coarse shadows,
  // FP32 coefficient copies (homogeneous boundary data)
  DBuf<float> E, F32, QC32, DeW32, DnS32, CC32, ID32, pcoef32, cfd32, bcg32, rpack32;
  // the smoother's packed operands (k_relax): per chunk and colour the face
  // coefficients -- on levels whose h^2 is a power of two pre-multiplied by
  // the exact 1/h^2 -- and InvDiagS; built on the host from these copies
  DBuf<double> rpack;
  DBuf<RelaxChunk> pchunks;        // chunk records with coefficient offsets (operand packing)
  DBuf<double> Uo, Uoo, fsrc;      // parabolic history (cells) and f staging
  bool f32_dirty = true;
  DecompH all_cells;               // every cell of every level (batch force reset)
  DecompH below_top;               // every cell of the levels below the finest
  bool update_fold = false;        // mixed form: Q += E may join the finest restriction (k_restrict_update)
  std::vector<InstRes> hir;        // host copy of the per-instance reduction plan
  // results of the last solve, per instance
  std::vector<double> res_hist;    // [ninst][hist_stride]
  std::vector<int> res_iters;
  std::vector<ResAcc> res_acc;
  DBuf<int8_t> g_type;
  DBuf<int> g_dst, g_a, g_b, g_c, g_d, g_e;
  // the fill that follows a restriction into the level (k_restrict_fill):
  // operands a, b, c of every ghost item, a cell under the finer level's
  // footprint coded -1 - (entry of ga_rt)
  DBuf<int> ga_a, ga_b, ga_c;
  DBuf<int2> ga_rt;
  // window tables for the prolongation fused with the parent's closing fill
  // (k_fill_prolong): a parent ghost cell coded -1 - (its ghost item)
  DBuf<int> win_alt;
  DBuf<PatchD> patches;
  DBuf<ResAcc> acc;
  DBuf<Rule> perim;                // per-patch perimeter ghost rules (inline)
  DBuf<RelaxChunkD> rchunks;       // relax chunk records as the kernels read them, all levels
  DBuf<uint8_t> cact;              // per chunk: its instance still iterates (batches, kActChunk)
  DBuf<int> crange;                // per instance and level: its chunk range [begin, end)
  int act_mode = 0;                // kActNone (one instance) / kActChunk (batch)
  DBuf<LevelX> levelx;             // per-level descriptors for the residual
  DBuf<ResTask> rtasks;            // residual warp tasks
  DBuf<InstRes> instres;           // per-instance residual reduction plan
  DBuf<SlotRange> sranges;
  DBuf<CoarsestD> coarsest;        // one coarsest operator per instance
  int nrtasks = 0, nslots = 0, npartials = 0, hist_stride = 0;
  ResAcc *acc_host = nullptr;      // ninst entries (pageable: freeing pinned memory synchronises the device)
  int *active_host = nullptr;      // ninst entries
  // graph of one V-cycle + fill-down + residual
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  // the whole solve loop on the device: a WHILE node around that iteration
  cudaGraph_t wgraph = nullptr;
  cudaGraphExec_t wexec = nullptr;
  bool while_tried = false;
  // the whole solve -- preamble and device-side loop -- as one graph
  cudaGraph_t sgraph = nullptr;
  cudaGraphExec_t sexec = nullptr;
  bool solve_tried = false;
  int64_t kernels_per_cycle = 0;
  // profiling
  bool profiling = false;
  int profile_level = 0;           // 0: every level
  struct Rec { int kind; cudaEvent_t a, b; double bytes; };
  std::vector<Rec> recs;
  int64_t launch_count = 0;
  int64_t graph_launches = 0;
  int64_t while_bodies = 0;        // iterations run inside WHILE graphs
  int64_t solve_graphs = 0;        // solves run as one graph launch
  int64_t preamble_kernels = 0;    // kernels of such a solve before its loop
  // per precision and level: colour cells per smoother thread (1, 2, 4),
  // picked by the autotuner at the first solve (result-neutral)
  std::vector<int> relax_n[2];
  bool tuned[2] = {false, false};
  DBuf<double> saveQ, saveQC, saveF;
};

namespace {

Fields fields(bsam_hier h) {
  Fields f;
  f.Q = h->Q.p; f.F = h->F.p; f.QC = h->QC.p;
  f.FTrue = h->FTrue.p; f.CC = h->CC.p; f.ID = h->ID.p; f.DeW = h->DeW.p; f.DnS = h->DnS.p;
  f.bcg = h->bcg.p; f.cfd = h->cfd.p; f.pcoef = h->pcoef.p; f.flags = h->flags.p;
  f.win = h->win.p; f.fp = h->fp.p; f.active = h->active.p;
  return f;
}

LevelD leveld(bsam_hier h, int k) {
  const LevelPlan &L = h->lev[k];
  LevelD d;
  d.patches = h->patches.p + L.p0;
  d.hx = L.hx; d.hy = L.hy;
  d.hx2 = L.hx * L.hx; d.hy2 = L.hy * L.hy;
  d.ihx2 = 1.0 / d.hx2; d.ihy2 = 1.0 / d.hy2;
  d.pow2 = L.pow2 ? 1 : 0;
  d.fhx = (float)d.hx; d.fhy = (float)d.hy; d.fhx2 = (float)d.hx2; d.fhy2 = (float)d.hy2;
  return d;
}

Decomp decomp(bsam_hier h, const DecompH &D) {
  Decomp d;
  d.beg = h->ints.p + D.beg_off;
  d.blk_p0 = h->ints.p + D.blk_off;
  d.n = D.n;
  d.nblocks = D.nblocks;
  return d;
}

inline int nblk(int n) { return (n + kBlock - 1) / kBlock; }

// kernels whose kBlock grid has fewer blocks than this run with 64-thread
// (or one-chunk) blocks: an SM issues about two FP64 operations per clock,
// so spreading a level's FP64 work over more SMs shortens the launch.  A
// batch keeps the larger blocks beyond two per SM: in its last V-cycles most
// instances are frozen and every extra block is scheduled for nothing.
int sm_count();
int spread_limit(bsam_hier h) { return (h->ninst > 1 ? 2 : 8) * sm_count(); }

// multiprocessors of the current device (queried once)
int sm_count() {
  static std::once_flag once;
  static int n = 152;
  std::call_once(once, [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
      n = v;
    cudaGetLastError();
  });
  return n;
}

// Every kernel goes out with programmatic stream serialization: the next
// kernel is scheduled while the previous one drains and waits for it at its
// griddepcontrol.wait (kernels.cuh chain_in).
template <typename... KArgs, typename... Args>
void launch_k(bsam_hier h, void (*kern)(KArgs...), int grid, int block, Args... args) {
  if (grid <= 0) return;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = h->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, args...);
}

// launch bookkeeping: optional per-kernel CUDA events for profiling
struct Launch {
  bsam_hier h;
  int kind;
  double bytes;
  cudaEvent_t a = nullptr, b = nullptr;
  bool rec = false;
  Launch(bsam_hier h_, int kind_, double bytes_, int level = 0) : h(h_), kind(kind_), bytes(bytes_) {
    h->launch_count++;
    rec = h->profiling && (h->profile_level == 0 || h->profile_level == level);
    if (rec) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, h->stream);
    }
  }
  ~Launch() {
    if (rec) {
      cudaEventRecord(b, h->stream);
      h->recs.push_back({kind, a, b, bytes});
    }
  }
};

enum { K_RELAX, K_GHOST, K_RESTRICT, K_RING, K_LOAD, K_CORR, K_PROLONG, K_COARSEST, K_RESID };

// ---------------------------------------------------------------------------
GhostItems ghost_items(bsam_hier h) {
  return GhostItems{h->g_type.p, h->g_dst.p, h->g_a.p, h->g_b.p, h->g_c.p, h->g_d.p, h->g_e.p,
                    h->ninst > 1 ? h->g_inst.p : nullptr};
}

// the arrays of the FP64 solve or of the FP32 correction cycle
template <class T> FieldsT<T> fields_t(bsam_hier h);
template <> Fields fields_t<double>(bsam_hier h) { return fields(h); }
template <> FieldsT<float> fields_t<float>(bsam_hier h) {
  FieldsT<float> f;
  f.Q = h->E.p; f.F = h->F32.p; f.QC = h->QC32.p;
  f.FTrue = h->FTrue.p; f.CC = h->CC32.p; f.ID = h->ID32.p; f.DeW = h->DeW32.p; f.DnS = h->DnS32.p;
  f.bcg = h->bcg32.p; f.cfd = h->cfd32.p; f.pcoef = h->pcoef32.p; f.flags = h->flags.p;
  f.win = h->win.p; f.fp = h->fp.p; f.active = h->active.p;
  return f;
}

// the smoother's packed operands in the cycle's value type
template <class T> const T *relax_pack(bsam_hier h);
template <> const double *relax_pack<double>(bsam_hier h) { return h->rpack.p; }
template <> const float *relax_pack<float>(bsam_hier h) { return h->rpack32.p; }

// pack the smoother's operands of every chunk and colour (see kPackRows) on
// the device, from the resident DeW, DnS and InvDiagS: at upload and after
// any of the three changes
int build_relax_pack(bsam_hier h) {
  const size_t nch = h->pchunks.n;
  int rc;
  if (!h->rpack.p && (rc = h->rpack.alloc(std::max<size_t>(nch, 1) * 2 * kPackRows * kChunk))) return rc;
  for (int k = 1; k <= h->nlev; ++k) {
    const LevelPlan &L = h->lev[k];
    if (!L.rc_n) continue;
    const int64_t items = (int64_t)L.rc_n * 2 * kChunk;
    k_pack<<<(unsigned)((items + kBlock - 1) / kBlock), kBlock, 0, h->stream>>>(
        h->pchunks.p + L.rc_off, L.rc_n, h->DeW.p, h->DnS.p, h->ID.p, 1.0 / (L.hx * L.hx), 1.0 / (L.hy * L.hy),
        L.pow2 ? 1 : 0, h->rpack.p + (size_t)L.rc_off * 2 * kPackRows * kChunk);
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->stream));
  h->f32_dirty = true;
  return BSAM_OK;
}

// algorithmic bytes scale with the value type (FP64 figures x size/8)
template <class T> constexpr double tscale() { return (double)sizeof(T) / 8.0; }

// ghost fill of level k; `need` > 0 restricts a batch's fill to the
// instances that have level `need` (the fill after restricting level need)
template <class T = double>
void launch_fill(bsam_hier h, int k, int need = 0) {
  const LevelPlan &L = h->lev[k];
  if (!L.g1_n) return;
  FieldsT<T> f = fields_t<T>(h);
  Launch l(h, K_GHOST, 0, k);
  if (nblk(L.g1_n) < spread_limit(h))
    launch_k(h, k_ghost<T, 64>, (L.g1_n + 63) / 64, 64, ghost_items(h), L.g1_off, L.g1_n, f.Q, f.QC, f.bcg, L.hx,
             L.hy, (const int *)h->active.p, (const int *)h->inst_nlev.p, need);
  else
    launch_k(h, k_ghost<T>, nblk(L.g1_n), kBlock, ghost_items(h), L.g1_off, L.g1_n, f.Q, f.QC, f.bcg, L.hx, L.hy,
             (const int *)h->active.p, (const int *)h->inst_nlev.p, need);
}

// can the device co-schedule one cluster of `ctas` CTAs of kClusterBlock
// threads of this smoother variant (sizes above 8 are non-portable)
template <class T, bool kPow2>
bool cluster_fits(int ctas) {
  cudaFuncSetAttribute(k_relax_cluster<T, kPow2>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)ctas);
  cfg.blockDim = dim3(kClusterBlock);
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)ctas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  const cudaError_t e = cudaOccupancyMaxActiveClusters(&n, k_relax_cluster<T, kPow2>, &cfg);
  cudaGetLastError();
  return e == cudaSuccess && n >= 1;
}

// CTAs of the smoother's single-cluster launch: 16 where every variant fits,
// else 8, else 0 (the variant is then never chosen)
int cluster_ctas() {
  static std::once_flag once;
  static int cached = 0;
  std::call_once(once, [] {
    for (int c : {16, 8})
      if (cluster_fits<double, true>(c) && cluster_fits<double, false>(c) && cluster_fits<float, true>(c) &&
          cluster_fits<float, false>(c)) {
        cached = c;
        break;
      }
  });
  return cached;
}

// resident blocks of the persistent smoother on the whole device
template <class T, bool kPow2>
int persistent_blocks() {
  static std::once_flag once;
  static int cached = 1;
  std::call_once(once, [] {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_relax_p<T, kPow2>, kBlock, 0);
    cudaGetLastError();
    cached = std::max(1, sms * std::max(per, 1));
  });
  return cached;
}

template <class T, bool kPow2, class... Args>
void launch_cluster(bsam_hier h, int ctas, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)ctas);
  cfg.blockDim = dim3(kClusterBlock);
  cfg.stream = h->stream;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  at[1].id = cudaLaunchAttributeClusterDimension;
  at[1].val.clusterDim.x = (unsigned)ctas;
  at[1].val.clusterDim.y = 1;
  at[1].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  cudaLaunchKernelEx(&cfg, k_relax_cluster<T, kPow2>, args...);
}

// most shared memory per CTA of k_relax_dsm, and the amount for a slice of
// 2^shift elements (the slice, then ten values per thread)
constexpr int kDsmMaxBytes = 160 * 1024;
template <class T>
size_t dsm_smem(int shift) {
  return (((size_t)1 << shift) + 10 * (size_t)kDsmBlock) * sizeof(T);
}

// can the device co-schedule one cluster of `ctas` CTAs of k_relax_dsm with
// `smem` bytes of shared memory each (sets the kernel's attributes: any
// slice up to kDsmMaxBytes may be launched afterwards)
template <class T, bool kPow2>
bool dsm_fits(int ctas, size_t smem) {
  cudaFuncSetAttribute(k_relax_dsm<T, kPow2>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaFuncSetAttribute(k_relax_dsm<T, kPow2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kDsmMaxBytes);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)ctas);
  cfg.blockDim = dim3(kDsmBlock);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)ctas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  const cudaError_t e = cudaOccupancyMaxActiveClusters(&n, k_relax_dsm<T, kPow2>, &cfg);
  cudaGetLastError();
  return e == cudaSuccess && n >= 1;
}

// the slice size (log2, in elements) of k_relax_dsm on level k, or -1 where
// the level's Q range does not fit one cluster's shared memory or its chunks
// need more than one colour cell per thread
template <class T>
int dsm_shift_for(bsam_hier h, int k) {
  const int C = cluster_ctas();
  if (C <= 0) return -1;
  const LevelPlan &L = h->lev[k];
  if ((int64_t)L.rc_n * kChunk > (int64_t)C * kDsmBlock) return -1;
  const int64_t n = L.q_hi - L.q_lo, per = (n + C - 1) / C;
  int sh = 0;
  while (((int64_t)1 << sh) < per) ++sh;
  const size_t bytes = dsm_smem<T>(sh);
  if (bytes > (size_t)kDsmMaxBytes) return -1;
  const bool ok = L.pow2 ? dsm_fits<T, true>(C, bytes) : dsm_fits<T, false>(C, bytes);
  return ok ? sh : -1;
}

template <class T, bool kPow2, class... Args>
void launch_dsm(bsam_hier h, int ctas, size_t smem, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)ctas);
  cfg.blockDim = dim3(kDsmBlock);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = h->stream;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  at[1].id = cudaLaunchAttributeClusterDimension;
  at[1].val.clusterDim.x = (unsigned)ctas;
  at[1].val.clusterDim.y = 1;
  at[1].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  cudaLaunchKernelEx(&cfg, k_relax_dsm<T, kPow2>, args...);
}

// ebRelaxLevel (ebRelaxLevel.m:28-38): 2*nsweeps colour passes; the ghost
// refill after every colour is folded into the next pass (k_relax `fresh`),
// and one fill after the last pass leaves the ghost frame as the reference's.
// first_fresh: the first pass evaluates its neighbours' ghost rules too (the
// ghosts were not refilled since the interior last changed everywhere, and
// the rules give what a fill would)
template <class T = double>
void launch_relax(bsam_hier h, int k, int nsweeps, bool first_fresh = false, bool defer_fill = false) {
  if (nsweeps <= 0) return;
  const LevelPlan &L = h->lev[k];
  FieldsT<T> f = fields_t<T>(h);
  LevelD ld = leveld(h, k);
  const RelaxChunkD *ch = h->rchunks.p + L.rc_off;
  const T *pk = relax_pack<T>(h) + (size_t)L.rc_off * 2 * kPackRows * kChunk;
  const int grid = (L.rc_n + kBlock / kChunk - 1) / (kBlock / kChunk);
  const int unit = h->opts.omega == 1.0 ? 1 : 0;
  const uint8_t *ca = h->act_mode == kActChunk ? h->cact.p + L.rc_off : nullptr;
  const int am = h->act_mode;
  const std::vector<int> &rn = h->relax_n[sizeof(T) == sizeof(float) ? 1 : 0];
  const int kn = rn.empty() ? 1 : rn[k];
  if (kn == 5) {   // the whole relaxation (and its fill) in one cluster launch, solution in shared memory
    const int sh = L.dsm_shift[sizeof(T) == sizeof(float) ? 1 : 0];
    Launch l(h, K_RELAX, 24.0 * tscale<T>() * (double)L.ncells * 2 * nsweeps, k);
    const int C = cluster_ctas();
    const Rule *pr = (const Rule *)h->perim.p;
    const T om = (T)h->opts.omega;
    const int ff = first_fresh ? 1 : 0, gn = defer_fill ? 0 : L.g1_n;
    const size_t smem = dsm_smem<T>(sh);
    const int q0 = (int)L.q_lo, qn = (int)(L.q_hi - L.q_lo);
    if (L.pow2)
      launch_dsm<T, true>(h, C, smem, ld, ch, L.rc_n, f, pk, pr, om, unit, nsweeps, ff, ca, am, ghost_items(h),
                          L.g1_off, gn, L.hx, L.hy, q0, qn, sh);
    else
      launch_dsm<T, false>(h, C, smem, ld, ch, L.rc_n, f, pk, pr, om, unit, nsweeps, ff, ca, am, ghost_items(h),
                           L.g1_off, gn, L.hx, L.hy, q0, qn, sh);
    return;
  }
  if (kn == 0) {   // the whole relaxation and its fill in one cluster launch
    Launch l(h, K_RELAX, 24.0 * tscale<T>() * (double)L.ncells * 2 * nsweeps, k);
    const int C = cluster_ctas();
    const Rule *pr = (const Rule *)h->perim.p;
    const T om = (T)h->opts.omega;
    const int ff = first_fresh ? 1 : 0;
    if (L.pow2)
      launch_cluster<T, true>(h, C, ld, ch, L.rc_n, f, pk, pr, om, unit, nsweeps, ff, ca, am, ghost_items(h), L.g1_off,
                              L.g1_n, L.hx, L.hy);
    else
      launch_cluster<T, false>(h, C, ld, ch, L.rc_n, f, pk, pr, om, unit, nsweeps, ff, ca, am, ghost_items(h),
                               L.g1_off, L.g1_n, L.hx, L.hy);
    return;
  }
  for (int s = 0; s < nsweeps; ++s)
    for (int m = 0; m < 2; ++m) {
      const int fresh = (first_fresh || s > 0 || m > 0) ? 1 : 0;
      Launch l(h, K_RELAX, 24.0 * tscale<T>() * (double)L.ncells, k);
      if (kn == 3) {   // persistent blocks walking the chunk groups
        const Rule *pr = (const Rule *)h->perim.p;
        const T om = (T)h->opts.omega;
        if (L.pow2)
          launch_k(h, k_relax_p<T, true>, std::min(grid, persistent_blocks<T, true>()), kBlock, ld, ch, L.rc_n, f, pk,
                   pr, m, om, unit, fresh, ca, am);
        else
          launch_k(h, k_relax_p<T, false>, std::min(grid, persistent_blocks<T, false>()), kBlock, ld, ch, L.rc_n, f,
                   pk, pr, m, om, unit, fresh, ca, am);
        continue;
      }
      if (kn > 1) {
        const int cpb = kBlock * kn / kChunk;     // chunks per block
        const int g = (L.rc_n + cpb - 1) / cpb;
        const Rule *pr = (const Rule *)h->perim.p;
        const T om = (T)h->opts.omega;
        if (kn == 2) {
          if (L.pow2) launch_k(h, k_relax_n<T, true, 2>, g, kBlock, ld, ch, L.rc_n, f, pk, pr, m, om, unit, fresh, ca, am);
          else launch_k(h, k_relax_n<T, false, 2>, g, kBlock, ld, ch, L.rc_n, f, pk, pr, m, om, unit, fresh, ca, am);
        } else {
          if (L.pow2) launch_k(h, k_relax_n<T, true, 4>, g, kBlock, ld, ch, L.rc_n, f, pk, pr, m, om, unit, fresh, ca, am);
          else launch_k(h, k_relax_n<T, false, 4>, g, kBlock, ld, ch, L.rc_n, f, pk, pr, m, om, unit, fresh, ca, am);
        }
        continue;
      }
      // one chunk per block, the FP64 work over more SMs; the FP32 pass has
      // little arithmetic, and fewer, larger blocks schedule faster once the
      // level fills the SMs (starfish FP32 iteration 337 -> 326 us)
      const int lim = sizeof(T) == sizeof(float) ? sm_count() : spread_limit(h);
      if (grid < lim) {
        if (L.pow2)
          launch_k(h, k_relax<T, true, kChunk>, L.rc_n, kChunk, ld, ch, L.rc_n, f, pk, (const Rule *)h->perim.p, m,
                   (T)h->opts.omega, unit, fresh, ca, am);
        else
          launch_k(h, k_relax<T, false, kChunk>, L.rc_n, kChunk, ld, ch, L.rc_n, f, pk, (const Rule *)h->perim.p, m,
                   (T)h->opts.omega, unit, fresh, ca, am);
        continue;
      }
      if (L.pow2)
        launch_k(h, k_relax<T, true>, grid, kBlock, ld, ch, L.rc_n, f, pk, (const Rule *)h->perim.p, m,
                 (T)h->opts.omega, unit, fresh, ca, am);
      else
        launch_k(h, k_relax<T, false>, grid, kBlock, ld, ch, L.rc_n, f, pk, (const Rule *)h->perim.p, m,
                 (T)h->opts.omega, unit, fresh, ca, am);
    }
  if (!defer_fill) launch_fill<T>(h, k);
}

template <class T = double>
void launch_restrict(bsam_hier h, int k, int to_parent) {
  const LevelPlan &L = h->lev[k];
  Decomp D = decomp(h, L.coarse);
  Launch l(h, K_RESTRICT, 12.0 * tscale<T>() * (double)L.ncells, k);
  if (D.nblocks < spread_limit(h))
    launch_k(h, k_restrict<T, 64>, (D.n + 63) / 64, 64, leveld(h, k), D, fields_t<T>(h), to_parent);
  else
    launch_k(h, k_restrict<T>, D.nblocks, kBlock, leveld(h, k), D, fields_t<T>(h), to_parent);
}

// restriction of level k into QC and level k-1, then the ghost fill of
// level k-1 (launch_restrict + launch_fill(k - 1, k)) in one launch.  With
// fill_k, level k's own fill that precedes them (launch_fill(k)) joins the
// launch too: FILL_PRE after the pre-smoothing (ring items left out), FILL_TOP
// before the fill-down; the caller checks the level's fuse_pre / fuse_top.
// FILL_ZERO: the FP32 correction cycle's pre-smoothing fill on any level,
// its parent-level operands taken as the 0 they hold (k_restrict_fill).
// The parent's fill skips the instances without level k (need = k) unless
// need = 0 is given.
enum { FILL_NONE = 0, FILL_PRE = 1, FILL_TOP = 2, FILL_ZERO = 3 };

template <class T = double>
void launch_restrict_fill(bsam_hier h, int k, int fill_k = FILL_NONE, int need = -1) {
  if (need < 0) need = k;
  const LevelPlan &L = h->lev[k], &Lc = h->lev[k - 1];
  if (!Lc.g1_n) {
    if (fill_k) launch_fill<T>(h, k);
    launch_restrict<T>(h, k, 1);
    return;
  }
  Decomp D = decomp(h, L.coarse);
  FieldsT<T> f = fields_t<T>(h);
  Launch l(h, K_RESTRICT, 12.0 * tscale<T>() * (double)L.ncells, k);
  const GhostAlt A{h->ga_a.p, h->ga_b.p, h->ga_c.p, h->ga_rt.p};
  const int fn = fill_k ? L.g1_n : 0, fring = fill_k == FILL_TOP ? 1 : 0;
  // FILL_ZERO: the zero-parent form of the FP32 correction cycle
  const int zlo = fill_k == FILL_ZERO ? (int)L.q_lo : 0, zn = fill_k == FILL_ZERO ? (int)(L.q_hi - L.q_lo) : 0;
  if (nblk(D.n) + nblk(Lc.g1_n) + nblk(fn) < spread_limit(h)) {
    const int nb = (D.n + 63) / 64, nf = (fn + 63) / 64;
    launch_k(h, k_restrict_fill<T, 64>, nb + nf + (Lc.g1_n + 63) / 64, 64, leveld(h, k), D, f, 1, nb,
             ghost_items(h), A, Lc.g1_off, Lc.g1_n, Lc.hx, Lc.hy, (const int *)h->active.p,
             (const int *)h->inst_nlev.p, need, L.g1_off, fn, nf, fring, L.hx, L.hy, zlo, zn);
  } else {
    const int nb = nblk(D.n), nf = nblk(fn);
    launch_k(h, k_restrict_fill<T>, nb + nf + nblk(Lc.g1_n), kBlock, leveld(h, k), D, f, 1, nb, ghost_items(h), A,
             Lc.g1_off, Lc.g1_n, Lc.hx, Lc.hy, (const int *)h->active.p, (const int *)h->inst_nlev.p, need,
             L.g1_off, fn, nf, fring, L.hx, L.hy, zlo, zn);
  }
}

CorrCSR corr_csr(bsam_hier h, const LevelPlan &L) {
  return CorrCSR{h->ct_cell.p + L.ct_off, h->ct_patch.p + L.ct_off, h->ct_beg.p + L.ct_off, h->ct_item.p, h->ct_j.p};
}

// ebTransfer 'ring' + ebCoarseLoad (ebVcycle.m:28-29) in one launch
template <class T = double>
void launch_coarse_load(bsam_hier h, int k) {
  const LevelPlan &L = h->lev[k];
  Decomp D = decomp(h, L.coarse);
  const int ntgt = h->opts.mass_correction ? L.ct_n : 0;
  Launch l(h, K_LOAD, 50.0 * tscale<T>() * (double)L.ncells, k);
  const int *ri = (const int *)(h->ninst > 1 ? h->ring_inst.p : nullptr);
  if (D.nblocks < spread_limit(h)) {   // spread the footprint's FP64 work over more SMs
    auto nb = [](int n) { return (n + 63) / 64; };
    launch_k(h, k_load<T, 64>, nb(L.ring_n) + nb(D.n) + nb(ntgt), 64, leveld(h, k), leveld(h, k - 1), D,
             fields_t<T>(h), (const int *)h->ring.p, ri, L.ring_off, L.ring_n, corr_csr(h, L), ntgt);
  } else {
    launch_k(h, k_load<T>, nblk(L.ring_n) + D.nblocks + nblk(ntgt), kBlock, leveld(h, k), leveld(h, k - 1), D,
             fields_t<T>(h), (const int *)h->ring.p, ri, L.ring_off, L.ring_n, corr_csr(h, L), ntgt);
  }
}

template <class T = double>
void launch_prolong(bsam_hier h, int k, int correct) {
  const LevelPlan &L = h->lev[k];
  Decomp D = decomp(h, L.coarse);
  Launch l(h, K_PROLONG, 20.0 * tscale<T>() * (double)L.ncells, k);
  if (D.nblocks < spread_limit(h))
    launch_k(h, k_prolong<T, 64>, (D.n + 63) / 64, 64, leveld(h, k), D, fields_t<T>(h), correct);
  else
    launch_k(h, k_prolong<T>, D.nblocks, kBlock, leveld(h, k), D, fields_t<T>(h), correct);
}

// the closing fill of level k-1 and the prolongation-correction of level k
// (launch_fill(k - 1) + launch_prolong(k, 1)) in one launch
template <class T = double>
void launch_fill_prolong(bsam_hier h, int k) {
  const LevelPlan &L = h->lev[k], &Lc = h->lev[k - 1];
  if (!Lc.g1_n) {
    launch_prolong<T>(h, k, 1);
    return;
  }
  Decomp D = decomp(h, L.coarse);
  FieldsT<T> f = fields_t<T>(h);
  Launch l(h, K_PROLONG, 20.0 * tscale<T>() * (double)L.ncells, k);
  const WindowGhosts<T> W{h->win_alt.p, ghost_items(h), f.bcg, (T)Lc.hx, (T)Lc.hy};
  if (nblk(Lc.g1_n) + D.nblocks < spread_limit(h)) {
    const int nb = (Lc.g1_n + 63) / 64;
    launch_k(h, k_fill_prolong<T, 64>, nb + (D.n + 63) / 64, 64, ghost_items(h), Lc.g1_off, Lc.g1_n, nb,
             leveld(h, k), D, f, 1, W, (const int *)h->active.p, (const int *)h->inst_nlev.p);
  } else {
    const int nb = nblk(Lc.g1_n);
    launch_k(h, k_fill_prolong<T>, nb + D.nblocks, kBlock, ghost_items(h), Lc.g1_off, Lc.g1_n, nb, leveld(h, k), D,
             f, 1, W, (const int *)h->active.p, (const int *)h->inst_nlev.p);
  }
}

// the smoother's launch form of level k in the cycle's precision (1 before
// the autotuner ran)
template <class T>
int relax_form(bsam_hier h, int k) {
  const std::vector<int> &rn = h->relax_n[sizeof(T) == sizeof(float) ? 1 : 0];
  return rn.empty() ? 1 : rn[k];
}

// can level k's V-cycle leave its closing fill to the prolongation of level
// k + 1 (launch_fill_prolong): in the FP32 correction cycle, unless the
// post-smoothing runs as one cluster launch, which fills the level itself.
// The FP64 cycle keeps separate launches: there the fused launch's
// prolongation items wait for the parent ghosts' rules on top of their FP64
// work, and the starfish iteration measured no faster fused (the FP32 cycle
// 1% faster); both forms give the same bits.
template <class T>
bool fill_deferrable(bsam_hier h, int k) {
  if (sizeof(T) == sizeof(double)) return false;
  if (k == 1 || h->opts.npost <= 0) return true;
  return relax_form<T>(h, k) != 0;
}

// the FP32 correction cycle solves a homogeneous problem: no boundary rhs
template <class T = double>
void launch_coarsest(bsam_hier h, bool defer_fill = false) {
  {
    Launch l(h, K_COARSEST, 8.0 * (double)h->Ainv.n, 1);
    cudaLaunchConfig_t cfg = {};
    const int rows = h->ninst > 1 ? 8 : 1;
    cfg.gridDim = dim3((unsigned)((h->coarse_max_rows + rows - 1) / rows), (unsigned)h->ncoarse_patches);
    cfg.blockDim = dim3(32 * rows);
    cfg.stream = h->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const double *rhs = sizeof(T) == sizeof(double) ? (const double *)h->bcRhs.p : nullptr;
    if (rows == 1)
      cudaLaunchKernelEx(&cfg, k_coarsest<T, 1>, (const double *)h->Ainv.p, rhs, (const CoarsestD *)h->coarsest.p,
                         fields_t<T>(h));
    else
      cudaLaunchKernelEx(&cfg, k_coarsest<T, 8>, (const double *)h->Ainv.p, rhs, (const CoarsestD *)h->coarsest.p,
                         fields_t<T>(h));
  }
  if (!defer_fill) launch_fill<T>(h, 1);
}

// ebVcycle (ebVcycle.m:16-35) from level k down.  defer_fill: the caller
// fuses this level's closing fill with its own prolongation
template <class T = double>
void launch_vcycle(bsam_hier h, int k, bool defer_fill = false) {
  if (k == 1) {
    launch_coarsest<T>(h, defer_fill);
    return;
  }
  // the pre-smoothing's closing fill joins the restriction's launch where
  // upload proved that exact (fuse_pre) and on every level of the FP32
  // cycle (FILL_ZERO), unless the relaxation runs as k_relax_cluster, which
  // fills the level itself
  const bool zero = sizeof(T) == sizeof(float) && h->lev[k].range_own;
  const bool pre_fused = h->opts.npre > 0 && relax_form<T>(h, k) != 0 && (zero || h->lev[k].fuse_pre);
  launch_relax<T>(h, k, h->opts.npre, false, pre_fused);
  launch_restrict_fill<T>(h, k, !pre_fused ? FILL_NONE : zero ? FILL_ZERO : FILL_PRE);
  launch_coarse_load<T>(h, k);
  const bool fused = fill_deferrable<T>(h, k - 1);
  launch_vcycle<T>(h, k - 1, fused);
  if (fused) launch_fill_prolong<T>(h, k);
  else launch_prolong<T>(h, k, 1);
  // the fill after the correction (ebVcycle.m:32) only feeds the first
  // post-smoothing pass, whose ghost reads then evaluate the same rules on
  // the same cells; the fill after the smoothing leaves the frame as the
  // reference's
  if (h->opts.npost > 0) {
    launch_relax<T>(h, k, h->opts.npost, true, defer_fill);
  } else if (!defer_fill) {
    launch_fill<T>(h, k);
  }
}

// ebTransfer 'filldown' (ebTransfer.m:73-79); top_fill: the finest level's
// closing fill (left to it by launch_vcycle) joins the first launch
void launch_filldown(bsam_hier h, bool top_fill = false) {
  for (int kk = h->nlev; kk >= 2; --kk) launch_restrict_fill(h, kk, top_fill && kk == h->nlev ? FILL_TOP : FILL_NONE);
}

bool mixed(bsam_hier h) { return h->opts.precision == 1; }

// ebCompResidual (ebCompResidual.m:15-85): one launch over every level of
// every instance, then the per-instance reduction and stop test (mode 0:
// before the first V-cycle, 1: after one, 2: report only).  The mixed form
// also stores r (FP32) as the right-hand side of the next correction cycle.
void launch_residual(bsam_hier h, int mode) {
  double bytes = 0;
  for (int k = 1; k <= h->nlev; ++k) bytes += 41.0 * (double)h->lev[k].ncells;
  {
    Launch l(h, K_RESID, bytes);
    const int g256 = (h->nrtasks + kBlock / 32 - 1) / (kBlock / 32);
    if (g256 < spread_limit(h))
      launch_k(h, k_residual<64>, (h->nrtasks + 1) / 2, 64, (const LevelX *)h->levelx.p, (const PatchD *)h->patches.p,
               (const ResTask *)h->rtasks.p, h->nrtasks, fields(h), (const int *)h->ring.p, h->slots.p, h->nslots,
               h->opts.mass_correction, mixed(h) ? h->F32.p : (float *)nullptr);
    else
      launch_k(h, k_residual<>, g256, kBlock, (const LevelX *)h->levelx.p, (const PatchD *)h->patches.p,
               (const ResTask *)h->rtasks.p, h->nrtasks, fields(h), (const int *)h->ring.p, h->slots.p, h->nslots,
               h->opts.mass_correction, mixed(h) ? h->F32.p : (float *)nullptr);
  }
  Launch l(h, K_RESID, 0);
  launch_k(h, k_residual_final, h->ninst, kFinal, (const InstRes *)h->instres.p, (const SlotRange *)h->sranges.p,
           (const double *)h->slots.p, h->nslots, h->acc.p, h->active.p, h->iters.p, h->hist.p, h->hist_stride, mode,
           (const int *)h->crange.p, h->nlev, h->act_mode == kActChunk ? h->cact.p : nullptr);
}

// Ghost fills of several levels in one launch (k_ghost_spans); `lv` lists
// the levels in increasing order, none reading a ghost cell another of them
// writes.
template <class T = double>
void launch_fill_spans(bsam_hier h, const std::vector<int> &lv) {
  GhostSpans S{};
  int tot = 0, last = 0;
  for (int k : lv) {
    const LevelPlan &L = h->lev[k];
    if (!L.g1_n) continue;
    S.off[S.n] = L.g1_off;
    S.beg[S.n] = tot;
    S.hx[S.n] = L.hx;
    S.hy[S.n] = L.hy;
    tot += L.g1_n;
    last = k;
    ++S.n;
  }
  if (S.n == 0) return;
  if (S.n == 1) {
    launch_fill<T>(h, last);
    return;
  }
  S.beg[S.n] = tot;
  FieldsT<T> f = fields_t<T>(h);
  Launch l(h, K_GHOST, 0, last);
  if (nblk(tot) < spread_limit(h))
    launch_k(h, k_ghost_spans<T, 64>, (tot + 63) / 64, 64, ghost_items(h), S, f.Q, f.QC, f.bcg,
             (const int *)h->active.p);
  else
    launch_k(h, k_ghost_spans<T>, nblk(tot), kBlock, ghost_items(h), S, f.Q, f.QC, f.bcg, (const int *)h->active.p);
}

// Mixed form: after Q changed on every level at once (or before the first
// correction, when a new level's parent still holds its old values under
// the footprint), restrict finest first, then refill the ghosts coarsest
// first, so every fill reads parent cells (ghosts included) that are up to
// date and the composite residual sees a consistent hierarchy.  Launches:
// the fill of level k-1 joins the restriction from level k (its operands
// under level k's footprint restricted by the items, k_restrict_fill) where
// level k-1 is the root or its rules read no cell that a later restriction
// or fill writes (fuse_top); the other levels' fills follow the
// restrictions, several levels per launch where none reads a ghost cell of
// the level below it in the same launch.  The same values as one launch per
// restriction and per level's fill.
// whether launch_consistent starts with a plain restriction of the finest
// level (which k_restrict_update can run together with Q += E)
bool consistent_starts_plain(bsam_hier h) {
  const int n = h->nlev;
  return n >= 2 && !h->lev[n].fuse_top && n - 1 != 1 && !h->lev[n - 1].fuse_top;
}

// top_restricted: the finest level's restriction already ran
// (k_restrict_update; consistent_starts_plain holds)
void launch_consistent(bsam_hier h, bool top_restricted = false) {
  std::vector<int> rest;   // levels filled after the restrictions
  const bool top = h->nlev >= 2 && h->lev[h->nlev].fuse_top;
  if (!top) rest.push_back(h->nlev);
  for (int kk = h->nlev; kk >= 2; --kk) {
    const int p = kk - 1, own = top && kk == h->nlev ? FILL_TOP : FILL_NONE;
    if (p == 1 || h->lev[p].fuse_top) {
      launch_restrict_fill(h, kk, own, 0);
    } else {
      if (own) launch_fill(h, kk);
      if (!(top_restricted && kk == h->nlev)) launch_restrict(h, kk, 1);
      rest.push_back(p);
    }
  }
  std::sort(rest.begin(), rest.end());
  std::vector<int> grp;
  for (int k : rest) {
    if (!grp.empty() && ((grp.back() == k - 1 && h->lev[k].reads_pg) || (int)grp.size() == kMaxSpans)) {
      launch_fill_spans(h, grp);
      grp.clear();
    }
    grp.push_back(k);
  }
  launch_fill_spans(h, grp);
}

// F = FTrue (ebSolveCycles.m:30-34), once before a run of FP64 V-cycles
// instead of at the start of each: within a solve F is written only by the
// coarse loads, over the parent footprint (recomputed every V-cycle before
// any read) and at the flux-correction targets, whose value the load forms
// from FTrue itself (load_corr_item); every other cell keeps FTrue.  So the
// F each V-cycle reads is the one the reference's per-cycle reset gives.
void reset_force(bsam_hier h) {
  if (h->ninst == 1) {
    cudaMemcpyAsync(h->F.p, h->FTrue.p, sizeof(double) * h->n_cells, cudaMemcpyDeviceToDevice, h->stream);
  } else {
    Decomp D = decomp(h, h->all_cells);
    Launch l(h, K_LOAD, 16.0 * (double)h->n_cells);
    launch_k(h, k_freset, D.nblocks, kBlock, D, (const PatchD *)h->patches.p, fields(h));
  }
}

// one ebSolveCycles iteration body (mode 1 inside ebSolveCycles, 2 for an
// eager V-cycle).  FP64: F = FTrue, V-cycle, fill-down, residual.  Mixed:
// the FP32 correction E = 0, one FP32 FAS V-cycle of E against the stored
// residual, Q += E in FP64, restriction and ghost fill in FP64, FP64
// residual.  The FP64 body expects F = FTrue off the footprints
// (reset_force before the first iteration).
int launch_iteration(bsam_hier h, int mode) {
  if (mixed(h)) {
    CK(cudaMemsetAsync(h->E.p, 0, sizeof(float) * h->E.n, h->stream));
    // the finest level's closing fill of E is left out: nothing reads the
    // correction's ghosts after the cycle (the update reads cells, the next
    // cycle starts from E = 0)
    launch_vcycle<float>(h, h->nlev, true);
    const bool fold = h->update_fold && consistent_starts_plain(h);
    if (fold) {   // Q += E with the finest level's restriction
      const LevelPlan &L = h->lev[h->nlev];
      Decomp D = decomp(h, L.coarse), Du = decomp(h, h->below_top);
      Launch l(h, K_RESTRICT, 20.0 * (double)h->n_cells);
      if (nblk(D.n) + Du.nblocks < spread_limit(h)) {
        const int nb = (D.n + 63) / 64;
        launch_k(h, k_restrict_update<64>, nb + (Du.n + 63) / 64, 64, leveld(h, h->nlev), D, fields(h),
                 (const float *)h->E.p, nb, Du, (const PatchD *)h->patches.p);
      } else {
        const int nb = nblk(D.n);
        launch_k(h, k_restrict_update<>, nb + Du.nblocks, kBlock, leveld(h, h->nlev), D, fields(h),
                 (const float *)h->E.p, nb, Du, (const PatchD *)h->patches.p);
      }
    } else {
      Decomp D = decomp(h, h->all_cells);
      Launch l(h, K_PROLONG, 20.0 * (double)h->n_cells);
      launch_k(h, k_update, D.nblocks, kBlock, D, (const PatchD *)h->patches.p, h->Q.p, (const float *)h->E.p,
               (const int *)h->active.p);
    }
    launch_consistent(h, fold);
    launch_residual(h, mode);
    CK(cudaGetLastError());
    return BSAM_OK;
  }
  // the finest level's closing fill joins the fill-down's first launch
  const bool top = h->nlev >= 2 && h->lev[h->nlev].fuse_top &&
                   (h->opts.npost <= 0 || relax_form<double>(h, h->nlev) != 0);
  launch_vcycle(h, h->nlev, top);
  launch_filldown(h, top);
  launch_residual(h, mode);
  CK(cudaGetLastError());
  return BSAM_OK;
}

// Autotuner of the smoother's launch form, per level and precision: on a
// level large enough to matter, 1, 2 or 4 colour cells per thread or the
// persistent form (kn 3: resident blocks walking the chunk groups); on a
// level that one thread-block cluster covers with at most 4 cells per
// thread, separate launches per colour pass or the single cluster launch
// (kn 0).  Each candidate's relaxation (npre sweeps and the closing fill) is
// timed best of three with CUDA events on the stream, in the precision the
// cycle runs in; the fastest is kept.  The choice does not change a single
// bit of the result (each update's arithmetic is the same), so it is tuned
// on the live state and the FP64 state is restored afterwards.
// BSAM_RELAX_N=0|1|2|3|4 forces one form on every level.
constexpr int64_t kTuneMinCells = 131072;
constexpr int kClusterMaxPerThread = 4;

// candidate set of a level: 0 none, 1 coarsening {1,2,4}, 2 {1, cluster}
int tune_set(bsam_hier h, int k) {
  const LevelPlan &L = h->lev[k];
  if (L.ncells >= kTuneMinCells) return 1;
  const int C = cluster_ctas();
  if (C > 0 && (int64_t)L.rc_n * kChunk <= (int64_t)kClusterMaxPerThread * C * kClusterBlock) return 2;
  return 0;
}

// microseconds of one relaxation of level k (npre sweeps and the fill) in
// launch form kn, timed as the solve runs it: a graph of kRelax relaxations
// in a row (a graph launch's own granularity then divides by kRelax); a
// form the runtime refuses is not a candidate (+inf)
template <class T>
float time_form(bsam_hier h, int k, int kn, int ns) {
  constexpr int kRelax = 8;
  std::vector<int> &rn = h->relax_n[sizeof(T) == sizeof(float) ? 1 : 0];
  rn[k] = kn;
  cudaGetLastError();
  if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return 1e30f;
  for (int r = 0; r < kRelax; ++r) launch_relax<T>(h, k, ns);
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
  float t = 1e30f;
  cudaEvent_t a = nullptr, b = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  if (e == cudaSuccess) e = cudaGraphLaunch(ge, h->stream);   // warm-up
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
    cudaEventRecord(a, h->stream);
    cudaGraphLaunch(ge, h->stream);
    cudaEventRecord(b, h->stream);
    e = cudaEventSynchronize(b);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    if (e == cudaSuccess) t = std::min(t, 1000.0f * ms / kRelax);
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (ge) cudaGraphExecDestroy(ge);
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();
  return e == cudaSuccess ? t : 1e30f;
}

template <class T>
int tune_level(bsam_hier h, int k, int set, int *best) {
  const int p = sizeof(T) == sizeof(float) ? 1 : 0;
  std::vector<int> &rn = h->relax_n[p];
  float bt = 1e30f;
  *best = 1;
  const int ns = std::max(h->opts.npre, 1);
  std::vector<int> cand = set == 1 ? std::vector<int>{1, 2, 4, 3} : std::vector<int>{1};
  if (set == 2) cand.push_back(0);
  h->lev[k].dsm_shift[p] = dsm_shift_for<T>(h, k);
  if (h->lev[k].dsm_shift[p] >= 0) cand.push_back(5);
  for (int kn : cand) {
    const float t = time_form<T>(h, k, kn, ns);
    if (t < bt * 0.97f) {              // a change must win clearly
      bt = t;
      *best = kn;
    }
  }
  rn[k] = *best;
  CK(cudaStreamSynchronize(h->stream));
  return BSAM_OK;
}

int autotune(bsam_hier h);

uint64_t tune_key(int precision, bool pow2, int chunks, int set) {
  int b = 0;
  while ((chunks >> (b + 1)) > 0) ++b;
  return ((uint64_t)set << 48) | ((uint64_t)precision << 40) | ((uint64_t)pow2 << 32) | (uint64_t)b;
}

// FP32 arrays of the mixed form: allocated on first use, coefficient copies
// refreshed whenever the FP64 coefficients changed
int ensure_f32(bsam_hier h) {
  if (!mixed(h)) return BSAM_OK;
  int rc;
  if (!h->E.p) {
    if ((rc = h->E.alloc(h->Q.n)) || (rc = h->F32.alloc(h->F.n)) || (rc = h->QC32.alloc(std::max<size_t>(h->QC.n, 1))) ||
        (rc = h->DeW32.alloc(h->DeW.n)) || (rc = h->DnS32.alloc(h->DnS.n)) || (rc = h->CC32.alloc(h->CC.n)) ||
        (rc = h->ID32.alloc(h->ID.n)) || (rc = h->pcoef32.alloc(std::max<size_t>(h->pcoef.n, 1))) ||
        (rc = h->cfd32.alloc(std::max<size_t>(h->cfd.n, 1))) || (rc = h->bcg32.alloc(std::max<size_t>(h->bcg.n, 1))) ||
        (rc = h->rpack32.alloc(h->rpack.n)))
      return rc;
    CK(cudaMemsetAsync(h->F32.p, 0, sizeof(float) * h->F32.n, h->stream));
    CK(cudaMemsetAsync(h->QC32.p, 0, sizeof(float) * h->QC32.n, h->stream));
    CK(cudaMemsetAsync(h->bcg32.p, 0, sizeof(float) * h->bcg32.n, h->stream));
    h->f32_dirty = true;
  }
  if (h->f32_dirty) {
    const std::pair<DBuf<double> *, DBuf<float> *> cv[] = {{&h->DeW, &h->DeW32}, {&h->DnS, &h->DnS32},
                                                           {&h->CC, &h->CC32},   {&h->ID, &h->ID32},
                                                           {&h->pcoef, &h->pcoef32}, {&h->cfd, &h->cfd32},
                                                           {&h->rpack, &h->rpack32}};
    for (const auto &c : cv)
      if (c.first->n) launch_k(h, k_to_f32, 4 * 152, kBlock, (const double *)c.first->p, c.second->p, (long long)c.first->n);
    CK(cudaGetLastError());
    h->f32_dirty = false;
  }
  return BSAM_OK;
}

int autotune(bsam_hier h) {
  const int p = mixed(h) ? 1 : 0;
  if (h->tuned[p]) return BSAM_OK;
  h->tuned[p] = true;
  std::vector<int> &rn = h->relax_n[p];
  rn.assign(h->nlev + 1, 1);
  // the shared-memory form only where the level's Q range fits one cluster
  auto dsm_ok = [&](int k) {
    const int sh = p ? dsm_shift_for<float>(h, k) : dsm_shift_for<double>(h, k);
    h->lev[k].dsm_shift[p] = sh;
    return sh >= 0;
  };
  if (const char *env = getenv("BSAM_RELAX_N")) {
    int kn = atoi(env);
    if (kn == 0 && cluster_ctas() == 0) kn = 1;
    rn.assign(h->nlev + 1, (kn >= 0 && kn <= 5) ? kn : 1);
    rn[1] = 1;
    for (int k = 2; k <= h->nlev; ++k)
      if (rn[k] == 5 && !dsm_ok(k)) rn[k] = 1;
    return BSAM_OK;
  }
  // levels already measured on this context (same precision, same h^2 form,
  // chunk count within a factor of two) take the cached choice
  bsam_ctx_s *c = h->ctx;
  std::vector<int> todo;
  {
    std::lock_guard<std::mutex> lk(c->tune_mu);
    for (int k = 2; k <= h->nlev; ++k) {
      const int set = tune_set(h, k);
      if (!set) continue;
      auto it = c->relax_tune.find(tune_key(p, h->lev[k].pow2, h->lev[k].rc_n, set));
      if (it != c->relax_tune.end()) rn[k] = it->second == 5 && !dsm_ok(k) ? 1 : it->second;
      else todo.push_back(k);
    }
  }
  if (todo.empty()) return BSAM_OK;
  // the FP64 smoother runs on the solution itself: keep a copy to put back
  // (the FP32 correction is zeroed at the start of every correction cycle)
  DBuf<double> keep;
  int rc = BSAM_OK;
  if (!p) {
    if ((rc = keep.alloc(h->Q.n))) return rc;
    CK(cudaMemcpyAsync(keep.p, h->Q.p, sizeof(double) * h->Q.n, cudaMemcpyDeviceToDevice, h->stream));
  }
  const bool prof = h->profiling;
  const int64_t lc = h->launch_count;
  h->profiling = false;
  for (int k : todo) {
    int best = 1;
    const int set = tune_set(h, k);
    rc = p ? tune_level<float>(h, k, set, &best) : tune_level<double>(h, k, set, &best);
    if (rc) break;
    std::lock_guard<std::mutex> lk(c->tune_mu);
    c->relax_tune[tune_key(p, h->lev[k].pow2, h->lev[k].rc_n, set)] = best;
  }
  h->profiling = prof;
  h->launch_count = lc;
  if (!p) {
    cudaError_t e = cudaMemcpyAsync(h->Q.p, keep.p, sizeof(double) * h->Q.n, cudaMemcpyDeviceToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    keep.release();
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, "autotune restore");
  }
  return rc;
}

int build_graph(bsam_hier h) {
  if (h->gexec) return BSAM_OK;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  const int64_t before = h->launch_count;
  int rc = launch_iteration(h, 1);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  h->kernels_per_cycle = h->launch_count - before;
  h->graph = g;
  CK(cudaGraphInstantiate(&h->gexec, g, 0));
  return BSAM_OK;
}

void drop_graph(bsam_hier h) {
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  if (h->graph) cudaGraphDestroy(h->graph);
  if (h->wexec) cudaGraphExecDestroy(h->wexec);
  if (h->wgraph) cudaGraphDestroy(h->wgraph);
  if (h->sexec) cudaGraphExecDestroy(h->sexec);
  if (h->sgraph) cudaGraphDestroy(h->sgraph);
  h->sexec = nullptr;
  h->sgraph = nullptr;
  h->solve_tried = false;
  h->gexec = nullptr;
  h->graph = nullptr;
  h->wexec = nullptr;
  h->wgraph = nullptr;
  h->while_tried = false;
}

// BSAM_SOLVE_LOOP=host selects the per-iteration graph with a host check of
// the stop tests instead of the device-side loop (the same kernels and
// results): profilers that cannot see the kernel nodes of a graph holding a
// conditional node (ncu) see every kernel of the solve that way
bool host_loop() {
  const char *e = getenv("BSAM_SOLVE_LOOP");
  return e && std::strcmp(e, "host") == 0;
}

// ebSolveCycles' loop as one graph: a conditional WHILE node whose body is
// one iteration followed by k_any_active, which sets the condition from the
// instances' stop tests.  A solve is then one graph launch and one read of
// the results, with no host round trip per V-cycle.  Returns false (and the
// per-iteration graph is used) when the runtime cannot build it.
bool build_while_graph(bsam_hier h) {
  if (h->wexec) return true;
  if (h->while_tried) return false;
  h->while_tried = true;
  cudaGraph_t g = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
  cudaGraphConditionalHandle cond;
  cudaGraphNodeParams np = {};
  cudaGraphNode_t node;
  bool ok = cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  if (ok) {
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np) == cudaSuccess;
  }
  if (ok) {
    cudaGraph_t body = np.conditional.phGraph_out[0];
    ok = cudaStreamBeginCaptureToGraph(h->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
         cudaSuccess;
    if (ok) {
      const int64_t before = h->launch_count;
      const int rc = launch_iteration(h, 1);
      h->kernels_per_cycle = h->launch_count - before;
      launch_k(h, k_any_active, 1, kBlock, (const int *)h->active.p, h->ninst, cond, cond, 0);
      cudaGraph_t out = nullptr;
      ok = cudaStreamEndCapture(h->stream, &out) == cudaSuccess && rc == BSAM_OK;
      h->launch_count = before;
    }
  }
  if (ok) ok = cudaGraphInstantiate(&h->wexec, g, 0) == cudaSuccess;
  cudaGetLastError();   // a refused build leaves no sticky error behind
  if (!ok) {
    if (h->wexec) cudaGraphExecDestroy(h->wexec);
    h->wexec = nullptr;
    cudaGraphDestroy(g);
    return false;
  }
  h->wgraph = g;
  return true;
}

// a conditional node after the capturing stream's current dependencies,
// whose body graph is captured from `body` (launches on the hierarchy's
// stream, redirected to a helper stream); the capture continues after it
bool add_conditional(bsam_hier h, cudaStream_t helper, cudaGraphConditionalHandle cond, cudaGraphConditionalNodeType ty,
                     const std::function<int()> &body) {
  cudaStreamCaptureStatus st;
  cudaGraph_t cg = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  if (cudaStreamGetCaptureInfo(h->stream, &st, nullptr, &cg, &deps, nullptr, &nd) != cudaSuccess ||
      st != cudaStreamCaptureStatusActive)
    return false;
  std::vector<cudaGraphNode_t> dv(deps, deps + nd);
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = cond;
  np.conditional.type = ty;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, cg, dv.data(), nullptr, dv.size(), &np) != cudaSuccess) return false;
  const cudaStream_t main = h->stream;
  h->stream = helper;
  bool ok = cudaStreamBeginCaptureToGraph(helper, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  int rc = BSAM_OK;
  if (ok) {
    rc = body();
    cudaGraph_t out = nullptr;
    ok = cudaStreamEndCapture(helper, &out) == cudaSuccess && rc == BSAM_OK;
  }
  h->stream = main;
  return ok && cudaStreamUpdateCaptureDependencies(main, &node, nullptr, 1, cudaStreamSetCaptureDependencies) ==
                   cudaSuccess;
}

// ebSolveCycles.m:8-70 as one graph: the preamble (F = FTrue, the ghost fill
// of every level, the initial residual and stop test; in the mixed form,
// while an instance iterates, the consistency step and the first
// correction's right-hand side) and then the device-side loop, so a solve
// is one graph launch and one read of the results.  Built once the smoother
// is tuned; returns false (and the step-by-step path is used) when the
// runtime cannot build it.
bool build_solve_graph(bsam_hier h) {
  if (h->sexec) return true;
  if (h->solve_tried) return false;
  h->solve_tried = true;
  cudaStream_t helper = nullptr;
  if (cudaStreamCreateWithFlags(&helper, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const int64_t before = h->launch_count;
  bool ok = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  cudaGraphConditionalHandle wcond = 0, icond = 0;
  if (ok) {
    cudaStreamCaptureStatus st;
    cudaGraph_t cg = nullptr;
    ok = cudaStreamGetCaptureInfo(h->stream, &st, nullptr, &cg, nullptr, nullptr, nullptr) == cudaSuccess &&
         cudaGraphConditionalHandleCreate(&wcond, cg, 1, cudaGraphCondAssignDefault) == cudaSuccess &&
         (!mixed(h) || cudaGraphConditionalHandleCreate(&icond, cg, 1, cudaGraphCondAssignDefault) == cudaSuccess);
    if (ok) {
      if (!mixed(h)) reset_force(h);
      for (int k = 1; k <= h->nlev; ++k) launch_fill(h, k);
      launch_residual(h, 0);
      launch_k(h, k_any_active, 1, kBlock, (const int *)h->active.p, h->ninst, wcond, icond, mixed(h) ? 1 : 0);
      h->preamble_kernels = h->launch_count - before;
      if (mixed(h))
        ok = add_conditional(h, helper, icond, cudaGraphCondTypeIf, [h]() {
          launch_consistent(h);
          launch_residual(h, 2);
          return cudaGetLastError() == cudaSuccess ? BSAM_OK : BSAM_ERR_CUDA;
        });
      if (ok)
        ok = add_conditional(h, helper, wcond, cudaGraphCondTypeWhile, [h, wcond]() {
          const int rc = launch_iteration(h, 1);
          launch_k(h, k_any_active, 1, kBlock, (const int *)h->active.p, h->ninst, wcond, wcond, 0);
          return rc;
        });
    }
    cudaGraph_t g = nullptr;
    const bool ended = cudaStreamEndCapture(h->stream, &g) == cudaSuccess;
    ok = ok && ended;
    if (ok) ok = cudaGraphInstantiate(&h->sexec, g, 0) == cudaSuccess;
    if (ok) h->sgraph = g;
    else if (g) cudaGraphDestroy(g);
  }
  h->launch_count = before;
  cudaStreamDestroy(helper);
  cudaGetLastError();   // a refused build leaves no sticky error behind
  if (!ok) {
    if (h->sexec) cudaGraphExecDestroy(h->sexec);
    h->sexec = nullptr;
  }
  return ok;
}

// per-instance residuals and active flags -> host (pinned); returns the
// number of instances still iterating
int read_state(bsam_hier h, int *nactive) {
  CK(cudaMemcpyAsync(h->acc_host, h->acc.p, sizeof(ResAcc) * h->ninst, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(h->active_host, h->active.p, sizeof(int) * h->ninst, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  int n = 0;
  for (int i = 0; i < h->ninst; ++i) n += h->active_host[i] != 0;
  *nactive = n;
  return BSAM_OK;
}

int read_residual(bsam_hier h, double out[5]) {
  int na;
  int rc = read_state(h, &na);
  if (rc) return rc;
  for (int i = 0; i < 5; ++i) out[i] = h->acc_host[0].out[i];
  return BSAM_OK;
}

// (re)size the per-instance history and upload the reduction plan after a
// change of the stop tests
int upload_stops(bsam_hier h) {
  int rc;
  int stride = 1;
  for (const InstRes &r : h->hir) stride = std::max(stride, r.max_vcycles + 1);
  if (stride != h->hist_stride || !h->hist.p) {
    h->hist.release();
    h->hist_stride = stride;
    if ((rc = h->hist.alloc((size_t)h->ninst * stride))) return rc;
  }
  // the graphs hold the reduction plan's and history's device addresses
  drop_graph(h);
  h->instres.release();
  if ((rc = h->instres.upload(h->hir.data(), h->hir.size(), h->stream))) return rc;
  CK(cudaStreamSynchronize(h->stream));
  return BSAM_OK;
}

int apply_opts(bsam_hier h) {
  for (InstRes &r : h->hir) {
    r.max_vcycles = h->opts.max_vcycles;
    r.rel_tol = h->opts.rel_tol;
  }
  return upload_stops(h);
}

// ---------------------------------------------------------------------------
// plan construction

// the Q cells ghost item i reads (its rule's operands; a physical corner
// reads those of its two face rules and an interior cell)
template <class BT>
void ghost_reads(const BT &B, int i, std::vector<int> &out) {
  switch (B.gt[i]) {
    case G_COPY: case G_NEUMANN: case G_RING: out.push_back(B.ga[i]); break;
    case G_DIRICHLET: out.insert(out.end(), {B.ga[i], B.gb[i]}); break;
    case G_LIF_CORNER: out.insert(out.end(), {B.ga[i], B.gc[i]}); break;
    case G_QIF: case G_LIF: out.insert(out.end(), {B.ga[i], B.gb[i], B.gc[i]}); break;
    case G_QIF_END: out.insert(out.end(), {B.ga[i], B.gb[i], B.gc[i], B.gd[i], B.ge[i]}); break;
    case G_PHYS_CORNER:
      ghost_reads(B, B.ga[i], out);
      ghost_reads(B, B.gb[i], out);
      out.push_back(B.gc[i]);
      break;
    default: break;
  }
}

struct Builder {
  bsam_hier h;
  const bsam_hier_desc *d;
  std::vector<int> ints;
  std::vector<int8_t> gt;
  std::vector<int> gdst, ga, gb, gc, gd, ge, gi;
  std::vector<Rule> perim;         // per patch: W(my) E(my) S(mx) N(mx) inline rule (type -1: physical)
  std::vector<RelaxChunk> chunks;  // relax chunk records
  std::vector<int> pe_off;         // per patch offset into perim
  std::vector<int> pinst;          // per patch instance

  const int32_t *P(int p) const { return d->patches + (size_t)p * PDN; }

  DecompH make_decomp(int p0, int p1, int kind) {
    // kind 0 colour cells, 1 cells, 2 coarse cells
    DecompH D;
    D.beg_off = (int)ints.size();
    int acc = 0;
    std::vector<int> beg;
    for (int p = p0; p < p1; ++p) {
      beg.push_back(acc);
      const int mx = P(p)[PD_MX], my = P(p)[PD_MY];
      acc += kind == 0 ? mx * my / 2 : kind == 1 ? mx * my : (mx / 2) * (my / 2);
    }
    beg.push_back(acc);
    ints.insert(ints.end(), beg.begin(), beg.end());
    D.n = acc;
    D.nblocks = nblk(acc);
    D.blk_off = (int)ints.size();
    int p = 0;
    for (int b = 0; b < D.nblocks; ++b) {
      const int g = b * kBlock;
      while (g >= beg[p + 1]) ++p;
      ints.push_back(p);
    }
    return D;
  }

  // ghost program of one level: final rule per ghost cell (stages 1-3 of
  // ebFillGhosts.m in order, later stages overriding), ring refresh items,
  // physical corners last
  int ghosts(int k, LevelPlan &L) {
    // dst -> index into tmp, over the Q range of this level's patches (a flat
    // index: a level has one rule slot per ghost cell)
    int64_t qlo = INT64_MAX, qhi = 0;
    for (int p = L.p0; p < L.p1; ++p) {
      const int32_t *r = P(p);
      qlo = std::min<int64_t>(qlo, r[PD_QOFF]);
      qhi = std::max<int64_t>(qhi, (int64_t)r[PD_QOFF] + (int64_t)(r[PD_MX] + 2) * (r[PD_MY] + 2));
    }
    if (qlo < 0 || qhi > d->n_q || qhi <= qlo) return fail(BSAM_ERR_ARG, "patch Q range outside Q");
    L.q_lo = qlo;
    L.q_hi = qhi;
    std::vector<int> slot((size_t)(qhi - qlo), -1);
    bool outside = false;
    auto rule_at = [&](int dst) -> int {
      if (dst < qlo || dst >= qhi) { outside = true; return -1; }
      return slot[(size_t)(dst - qlo)];
    };
    struct G { int8_t t; int dst, a, b, c, dd, e; int inst = 0; };
    std::vector<G> tmp, ringi, corners;
    int cur = 0;                  // instance of the patch being planned
    auto put = [&](G g) {
      g.inst = cur;
      if (g.dst < qlo || g.dst >= qhi) { outside = true; return; }
      int &sl = slot[(size_t)(g.dst - qlo)];
      if (sl < 0) {
        sl = (int)tmp.size();
        tmp.push_back(g);
      } else {
        tmp[sl] = g;
      }
    };
    const bool qif = h->opts.ghost_interp == 0;
    for (int p = L.p0; p < L.p1; ++p) {
      const int32_t *r = P(p);
      const int mx = r[PD_MX], my = r[PD_MY], cmx = mx / 2, cmy = my / 2;
      const int qo = r[PD_QOFF];
      cur = pinst[p];
      auto Q = [&](int i, int j) { return qo + (i - 1) + (j - 1) * (mx + 2); };
      // 1. coarse-fine: ring refresh + ebInterpCf
      bool any = false;
      for (int s = 0; s < 4; ++s) any |= (r[PD_FIW + s] != 0) || (r[PD_CCSW + s] == 3);
      if (k > 1 && any) {
        std::vector<int> qcsrc((size_t)(cmx + 2) * (cmy + 2), -1);
        for (int t = r[PD_RING0]; t < r[PD_RING1]; ++t) {
          const int src = d->ring[2 * t], dst = d->ring[2 * t + 1];
          const int loc = dst - r[PD_QCOFF];
          if (loc < 0 || loc >= (int)qcsrc.size()) return fail(BSAM_ERR_ARG, "ring destination outside QC");
          qcsrc[loc] = src;
          ringi.push_back({G_RING, dst, src, 0, 0, 0, 0, cur});
        }
        bool bad = false;
        auto QC = [&](int i, int j) {
          const int v = qcsrc[(i - 1) + (j - 1) * (cmx + 2)];
          if (v < 0) bad = true;
          return v;
        };
        const int *fint = r + PD_FIW;
        if (fint[0]) {
          if (qif) {
            for (int rho = 3; rho <= my - 1; rho += 2) put({G_QIF, Q(1, rho), Q(3, rho + 2), Q(2, rho + 1), QC(1, (rho + 1) / 2), 0, 0});
            for (int rho = 4; rho <= my; rho += 2) put({G_QIF, Q(1, rho), Q(3, rho - 2), Q(2, rho - 1), QC(1, (rho + 2) / 2), 0, 0});
            put({G_QIF_END, Q(1, my + 1), Q(3, my + 1), Q(2, my + 1), QC(1, cmy + 2), QC(1, cmy + 1), QC(1, cmy)});
            put({G_QIF_END, Q(1, 2), Q(3, 2), Q(2, 2), QC(1, 1), QC(1, 2), QC(1, 3)});
          } else {
            for (int rho = 3; rho <= my + 1; rho += 2) put({G_LIF, Q(1, rho), Q(2, rho), Q(2, rho - 1), QC(1, (rho + 1) / 2), 0, 0});
            for (int rho = 2; rho <= my; rho += 2) put({G_LIF, Q(1, rho), Q(2, rho), Q(2, rho + 1), QC(1, (rho + 2) / 2), 0, 0});
          }
        }
        if (fint[1]) {
          if (qif) {
            for (int rho = 3; rho <= my - 1; rho += 2) put({G_QIF, Q(mx + 2, rho), Q(mx, rho + 2), Q(mx + 1, rho + 1), QC(cmx + 2, (rho + 1) / 2), 0, 0});
            for (int rho = 4; rho <= my; rho += 2) put({G_QIF, Q(mx + 2, rho), Q(mx, rho - 2), Q(mx + 1, rho - 1), QC(cmx + 2, (rho + 2) / 2), 0, 0});
            put({G_QIF_END, Q(mx + 2, my + 1), Q(mx, my + 1), Q(mx + 1, my + 1), QC(cmx + 2, cmy + 2), QC(cmx + 2, cmy + 1), QC(cmx + 2, cmy)});
            put({G_QIF_END, Q(mx + 2, 2), Q(mx, 2), Q(mx + 1, 2), QC(cmx + 2, 1), QC(cmx + 2, 2), QC(cmx + 2, 3)});
          } else {
            for (int rho = 3; rho <= my + 1; rho += 2) put({G_LIF, Q(mx + 2, rho), Q(mx + 1, rho), Q(mx + 1, rho - 1), QC(cmx + 2, (rho + 1) / 2), 0, 0});
            for (int rho = 2; rho <= my; rho += 2) put({G_LIF, Q(mx + 2, rho), Q(mx + 1, rho), Q(mx + 1, rho + 1), QC(cmx + 2, (rho + 2) / 2), 0, 0});
          }
        }
        if (fint[2]) {
          if (qif) {
            for (int kap = 3; kap <= mx - 1; kap += 2) put({G_QIF, Q(kap, 1), Q(kap + 2, 3), Q(kap + 1, 2), QC((kap + 1) / 2, 1), 0, 0});
            for (int kap = 4; kap <= mx; kap += 2) put({G_QIF, Q(kap, 1), Q(kap - 2, 3), Q(kap - 1, 2), QC((kap + 2) / 2, 1), 0, 0});
            put({G_QIF_END, Q(mx + 1, 1), Q(mx + 1, 3), Q(mx + 1, 2), QC(cmx + 2, 1), QC(cmx + 1, 1), QC(cmx, 1)});
            put({G_QIF_END, Q(2, 1), Q(2, 3), Q(2, 2), QC(1, 1), QC(2, 1), QC(3, 1)});
          } else {
            for (int kap = 3; kap <= mx + 1; kap += 2) put({G_LIF, Q(kap, 1), Q(kap, 2), Q(kap - 1, 2), QC((kap + 1) / 2, 1), 0, 0});
            for (int kap = 2; kap <= mx; kap += 2) put({G_LIF, Q(kap, 1), Q(kap, 2), Q(kap + 1, 2), QC((kap + 2) / 2, 1), 0, 0});
          }
        }
        if (fint[3]) {
          if (qif) {
            for (int kap = 3; kap <= mx - 1; kap += 2) put({G_QIF, Q(kap, my + 2), Q(kap + 2, my), Q(kap + 1, my + 1), QC((kap + 1) / 2, cmy + 2), 0, 0});
            for (int kap = 4; kap <= mx; kap += 2) put({G_QIF, Q(kap, my + 2), Q(kap - 2, my), Q(kap - 1, my + 1), QC((kap + 2) / 2, cmy + 2), 0, 0});
            put({G_QIF_END, Q(mx + 1, my + 2), Q(mx + 1, my), Q(mx + 1, my + 1), QC(cmx + 2, cmy + 2), QC(cmx + 1, cmy + 2), QC(cmx, cmy + 2)});
            put({G_QIF_END, Q(2, my + 2), Q(2, my), Q(2, my + 1), QC(1, cmy + 2), QC(2, cmy + 2), QC(3, cmy + 2)});
          } else {
            for (int kap = 3; kap <= mx + 1; kap += 2) put({G_LIF, Q(kap, my + 2), Q(kap, my + 1), Q(kap - 1, my + 1), QC((kap + 1) / 2, cmy + 2), 0, 0});
            for (int kap = 2; kap <= mx; kap += 2) put({G_LIF, Q(kap, my + 2), Q(kap, my + 1), Q(kap + 1, my + 1), QC((kap + 2) / 2, cmy + 2), 0, 0});
          }
        }
        const int8_t ct = qif ? G_QIF : G_LIF_CORNER;
        if (r[PD_CCSW] == 3) put(qif ? G{ct, Q(1, 1), Q(3, 3), Q(2, 2), QC(1, 1), 0, 0} : G{ct, Q(1, 1), Q(2, 2), 0, QC(1, 1), 0, 0});
        if (r[PD_CCSE] == 3) put(qif ? G{ct, Q(mx + 2, 1), Q(mx, 3), Q(mx + 1, 2), QC(cmx + 2, 1), 0, 0} : G{ct, Q(mx + 2, 1), Q(mx + 1, 2), 0, QC(cmx + 2, 1), 0, 0});
        if (r[PD_CCNW] == 3) put(qif ? G{ct, Q(1, my + 2), Q(3, my), Q(2, my + 1), QC(1, cmy + 2), 0, 0} : G{ct, Q(1, my + 2), Q(2, my + 1), 0, QC(1, cmy + 2), 0, 0});
        if (r[PD_CCNE] == 3) put(qif ? G{ct, Q(mx + 2, my + 2), Q(mx, my), Q(mx + 1, my + 1), QC(cmx + 2, cmy + 2), 0, 0} : G{ct, Q(mx + 2, my + 2), Q(mx + 1, my + 1), 0, QC(cmx + 2, cmy + 2), 0, 0});
        if (bad) return fail(BSAM_ERR_ARG, "coarse-fine stencil reads a QC cell outside the gathered ring");
      }
      // 2. same-level copies
      for (int t = r[PD_SAME0]; t < r[PD_SAME1]; ++t) put({G_COPY, d->same[2 * t + 1], d->same[2 * t], 0, 0, 0, 0});
      // 3. physical faces and corners
      const int go = r[PD_BCGOFF];
      const int gW = go, gE = go + my, gS = go + 2 * my, gN = go + 2 * my + mx;
      for (int j = 2; j <= my + 1; ++j) {
        if (r[PD_BCW] == 1) put({G_DIRICHLET, Q(1, j), Q(2, j), Q(3, j), 0, 0, gW + j - 2});
        else if (r[PD_BCW] == 2) put({G_NEUMANN, Q(1, j), Q(2, j), 0, 0, 0, gW + j - 2});
        if (r[PD_BCE] == 1) put({G_DIRICHLET, Q(mx + 2, j), Q(mx + 1, j), Q(mx, j), 0, 0, gE + j - 2});
        else if (r[PD_BCE] == 2) put({G_NEUMANN, Q(mx + 2, j), Q(mx + 1, j), 0, 0, 0, gE + j - 2});
      }
      for (int i = 2; i <= mx + 1; ++i) {
        if (r[PD_BCS] == 1) put({G_DIRICHLET, Q(i, 1), Q(i, 2), Q(i, 3), 0, 0, gS + i - 2});
        else if (r[PD_BCS] == 2) put({G_NEUMANN, Q(i, 1), Q(i, 2), 1, 0, 0, gS + i - 2});
        if (r[PD_BCN] == 1) put({G_DIRICHLET, Q(i, my + 2), Q(i, my + 1), Q(i, my), 0, 0, gN + i - 2});
        else if (r[PD_BCN] == 2) put({G_NEUMANN, Q(i, my + 2), Q(i, my + 1), 1, 0, 0, gN + i - 2});
      }
      // physical corners: (face ghost + face ghost) - interior; the face
      // ghosts are referenced by their destination here and resolved to
      // rule indices once the level's rules are final
      if (r[PD_CCSW] == 1) corners.push_back({G_PHYS_CORNER, Q(1, 1), Q(2, 1), Q(1, 2), Q(2, 2), 0, 0, cur});
      if (r[PD_CCSE] == 1) corners.push_back({G_PHYS_CORNER, Q(mx + 2, 1), Q(mx + 1, 1), Q(mx + 2, 2), Q(mx + 1, 2), 0, 0, cur});
      if (r[PD_CCNW] == 1) corners.push_back({G_PHYS_CORNER, Q(1, my + 2), Q(2, my + 2), Q(1, my + 1), Q(2, my + 1), 0, 0, cur});
      if (r[PD_CCNE] == 1) corners.push_back({G_PHYS_CORNER, Q(mx + 2, my + 2), Q(mx + 1, my + 2), Q(mx + 2, my + 1), Q(mx + 1, my + 1), 0, 0, cur});
    }
    if (outside) return fail(BSAM_ERR_ARG, "ghost destination outside its level's patches");
    L.g1_off = (int)gt.size();
    for (G &g : corners) {
      if (rule_at(g.dst) >= 0) return fail(BSAM_ERR_ARG, "physical corner also written by another ghost stage");
      const int i1 = rule_at(g.a), i2 = rule_at(g.b);
      if (i1 < 0 || i2 < 0) return fail(BSAM_ERR_ARG, "physical corner next to a ghost without a rule");
      g.a = L.g1_off + i1;
      g.b = L.g1_off + i2;
    }
    auto emit = [&](const std::vector<G> &v) {
      for (const G &g : v) {
        gt.push_back(g.t); gdst.push_back(g.dst); ga.push_back(g.a); gb.push_back(g.b);
        gc.push_back(g.c); gd.push_back(g.dd); ge.push_back(g.e); gi.push_back(g.inst);
      }
    };
    emit(tmp);
    emit(ringi);
    emit(corners);
    L.g1_n = (int)gt.size() - L.g1_off;
    // perimeter rule table for the relaxation's ghost evaluation: every cell
    // of an internal face has a value rule (COPY/QIF/QIF_END/LIF)
    for (int p = L.p0; p < L.p1; ++p) {
      const int32_t *r = P(p);
      const int mx = r[PD_MX], my = r[PD_MY], qo = r[PD_QOFF];
      auto Q = [&](int i, int j) { return qo + (i - 1) + (j - 1) * (mx + 2); };
      pe_off[p] = (int)perim.size();
      auto add = [&](int side, int dst) -> bool {
        if (r[PD_BCW + side] != 0) { perim.push_back(Rule{-1, 0, 0, 0, 0, 0, 0, 0}); return true; }
        const int ri = rule_at(dst);
        if (ri < 0) return false;
        const G &g = tmp[ri];
        if (g.t != G_COPY && g.t != G_QIF && g.t != G_QIF_END && g.t != G_LIF) return false;
        // operand slots the rule does not read repeat its first operand (the
        // smoother loads all five before it looks at the kind)
        Rule R{g.t, g.a, g.b, g.c, g.dd, g.e, 0, 0};
        if (g.t == G_COPY) R.b = R.c = g.a;
        if (g.t != G_QIF_END) R.d = R.e = g.a;
        perim.push_back(R);
        return true;
      };
      bool ok = true;
      for (int j = 2; j <= my + 1; ++j) ok = ok && add(0, Q(1, j));
      for (int j = 2; j <= my + 1; ++j) ok = ok && add(1, Q(mx + 2, j));
      for (int i = 2; i <= mx + 1; ++i) ok = ok && add(2, Q(i, 1));
      for (int i = 2; i <= mx + 1; ++i) ok = ok && add(3, Q(i, my + 2));
      if (!ok) return fail(BSAM_ERR_ARG, "internal face ghost without an interpolation or copy rule at level " +
                                             std::to_string(k));
    }
    // relax chunks: the colour cells of each patch in pieces of kChunk
    L.rc_off = (int)chunks.size();
    for (int p = L.p0; p < L.p1; ++p) {
      const int32_t *r = P(p);
      const int ncol = r[PD_MX] * r[PD_MY] / 2;
      for (int s0 = 0; s0 < ncol; s0 += kChunk) {
        RelaxChunk c{};
        c.q_off = r[PD_QOFF]; c.c_off = r[PD_COFF]; c.dew_off = r[PD_DEWOFF]; c.dns_off = r[PD_DNSOFF];
        c.bcg_off = r[PD_BCGOFF]; c.pe_off = pe_off[p]; c.mx = r[PD_MX]; c.my = r[PD_MY];
        c.par0 = r[PD_PAR0]; c.s0 = s0; c.n = std::min(kChunk, ncol - s0); c.inst = pinst[p];
        for (int sd = 0; sd < 4; ++sd) c.bc[sd] = r[PD_BCW + sd];
        chunks.push_back(c);
      }
    }
    L.rc_n = (int)chunks.size() - L.rc_off;
    // every index must stay inside Q / QC / bcg
    for (int i = L.g1_off; i < L.g1_off + L.g1_n; ++i) {
      const int8_t t = gt[i];
      auto okq = [&](int v) { return v >= 0 && v < d->n_q; };
      bool ok = t == G_RING ? (gdst[i] >= 0 && gdst[i] < d->n_qc) : okq(gdst[i]);
      ok = ok && okq(ga[i]);
      if (t == G_PHYS_CORNER) {
        ok = gdst[i] >= 0 && gdst[i] < d->n_q && ga[i] >= L.g1_off && ga[i] < i && gb[i] >= L.g1_off && gb[i] < i &&
             okq(gc[i]);
        if (!ok) return fail(BSAM_ERR_ARG, "physical corner rule out of range at level " + std::to_string(k));
        continue;
      }
      if (t == G_QIF || t == G_QIF_END || t == G_LIF || t == G_DIRICHLET) ok = ok && okq(gb[i]);
      if (t == G_QIF || t == G_QIF_END || t == G_LIF || t == G_LIF_CORNER) ok = ok && okq(gc[i]);
      if (t == G_QIF_END) ok = ok && okq(gd[i]) && okq(ge[i]);
      if (t == G_DIRICHLET || t == G_NEUMANN) ok = ok && ge[i] >= 0 && ge[i] < d->n_bcg;
      if (!ok) return fail(BSAM_ERR_ARG, "ghost rule index out of range at level " + std::to_string(k));
    }
    return BSAM_OK;
  }
};

int validate(const bsam_hier_desc *d) {
  if (!d || d->nlev < 1 || d->root_idx < 1 || d->root_idx > d->nlev || d->npatch < 1)
    return fail(BSAM_ERR_ARG, "bad hierarchy header");
  if (!d->levels || !d->hs || !d->patches || !d->Q || !d->F || !d->FTrue || !d->CC || !d->InvDiagS || !d->DeW ||
      !d->DnS || !d->covered || !d->Ainv || !d->bcRhs)
    return fail(BSAM_ERR_ARG, "missing array");
  int expect_p = 0;
  for (int k = 1; k <= d->nlev; ++k) {
    const int32_t *L = d->levels + (size_t)(k - 1) * LDN;
    if (L[LD_P0] != expect_p || L[LD_P1] <= L[LD_P0] || L[LD_P1] > d->npatch)
      return fail(BSAM_ERR_ARG, "level patch ranges must tile the patch table");
    expect_p = L[LD_P1];
    if (!(d->hs[2 * (k - 1)] > 0) || !(d->hs[2 * (k - 1) + 1] > 0)) return fail(BSAM_ERR_ARG, "bad cell size");
  }
  if (expect_p != d->npatch) return fail(BSAM_ERR_ARG, "patch count mismatch");
  const int ninst = d->ninst > 1 ? d->ninst : 1;
  if (d->levels[LD_P1] - d->levels[LD_P0] != ninst)
    return fail(BSAM_ERR_ARG, "level 1 must hold one patch per instance");
  if (ninst > 1) {
    if (!d->patch_inst || !d->inst_root) return fail(BSAM_ERR_ARG, "batch without instance tables");
    for (int p = 0; p < d->npatch; ++p)
      if (d->patch_inst[p] < 0 || d->patch_inst[p] >= ninst) return fail(BSAM_ERR_ARG, "patch instance out of range");
    for (int i = 0; i < ninst; ++i) {
      if (d->inst_root[i] < 1 || d->inst_root[i] > d->nlev) return fail(BSAM_ERR_ARG, "instance root out of range");
      if (d->patch_inst[i] != i) return fail(BSAM_ERR_ARG, "level-1 patches must be in instance order");
    }
    // each level holds its patches instance by instance
    for (int k = 1; k <= d->nlev; ++k) {
      const int32_t *L = d->levels + (size_t)(k - 1) * LDN;
      for (int p = L[LD_P0] + 1; p < L[LD_P1]; ++p)
        if (d->patch_inst[p] < d->patch_inst[p - 1])
          return fail(BSAM_ERR_ARG, "batch patches of a level must be grouped by instance, in instance order");
    }
  }
  for (int p = 0; p < d->npatch; ++p) {
    const int32_t *r = d->patches + (size_t)p * PDN;
    const int64_t mx = r[PD_MX], my = r[PD_MY];
    const int k = r[PD_LEVEL];
    if (k < 1 || k > d->nlev || mx < 2 || my < 2 || (k > 1 && (mx % 2 || my % 2)))
      return fail(BSAM_ERR_ARG, "bad patch size at patch " + std::to_string(p));
    auto in = [](int64_t off, int64_t len, int64_t n) { return off >= 0 && off + len <= n; };
    bool ok = in(r[PD_QOFF], (mx + 2) * (my + 2), d->n_q) && in(r[PD_COFF], mx * my, d->n_cells) &&
              in(r[PD_DEWOFF], (mx + 1) * my, d->n_dew) && in(r[PD_DNSOFF], mx * (my + 1), d->n_dns) &&
              in(r[PD_BCGOFF], 2 * (mx + my), d->n_bcg) && in(r[PD_SAME0], r[PD_SAME1] - r[PD_SAME0], d->n_same);
    if (k > 1) {
      const int64_t cmx = mx / 2, cmy = my / 2;
      ok = ok && in(r[PD_QCOFF], (cmx + 2) * (cmy + 2), d->n_qc) && in(r[PD_CFDOFF], 2 * (cmx + cmy), d->n_cfd) &&
           in(r[PD_PCOFF], (cmx + 1) * cmy + cmx * (cmy + 1) + cmx * cmy, d->n_pcoef) &&
           in(r[PD_RING0], r[PD_RING1] - r[PD_RING0], d->n_ring) && in(r[PD_WIN0], (cmx + 2) * (cmy + 2), d->n_win) &&
           in(r[PD_FP0], cmx * cmy, d->n_fp) && in(r[PD_CORR0], 2 * (cmx + cmy), d->n_corr);
    }
    for (int s = 0; s < 4; ++s) ok = ok && r[PD_BCW + s] >= 0 && r[PD_BCW + s] <= 2;
    if (!ok) return fail(BSAM_ERR_ARG, "patch " + std::to_string(p) + ": offsets outside the flat arrays");
  }
  for (int64_t t = 0; t < d->n_same; ++t)
    if (d->same[2 * t] < 0 || d->same[2 * t] >= d->n_q || d->same[2 * t + 1] < 0 || d->same[2 * t + 1] >= d->n_q)
      return fail(BSAM_ERR_ARG, "same-level table index out of range");
  for (int64_t t = 0; t < d->n_ring; ++t)
    if (d->ring[2 * t] < 0 || d->ring[2 * t] >= d->n_q || d->ring[2 * t + 1] < 0 || d->ring[2 * t + 1] >= d->n_qc)
      return fail(BSAM_ERR_ARG, "ring table index out of range");
  for (int64_t t = 0; t < d->n_win; ++t)
    if (d->win[t] < 0 || d->win[t] >= d->n_q) return fail(BSAM_ERR_ARG, "window table index out of range");
  for (int64_t t = 0; t < d->n_fp; ++t)
    if (d->fp[2 * t] < 0 || d->fp[2 * t] >= d->n_q || d->fp[2 * t + 1] < 0 || d->fp[2 * t + 1] >= d->n_cells)
      return fail(BSAM_ERR_ARG, "footprint table index out of range");
  for (int64_t t = 0; t < d->n_corr; ++t)
    if (d->corr[t] < -1 || d->corr[t] >= d->n_cells) return fail(BSAM_ERR_ARG, "correction target out of range");
  int64_t nc = 0;
  for (int i = 0; i < ninst; ++i) {
    const int32_t *r1 = d->patches + (size_t)i * PDN;
    if ((int64_t)r1[PD_MX] * r1[PD_MY] > 16384) return fail(BSAM_ERR_ARG, "coarsest level too large");
    nc += (int64_t)r1[PD_MX] * r1[PD_MY];
  }
  if (nc != d->ncoarse) return fail(BSAM_ERR_ARG, "coarsest size mismatch");
  return BSAM_OK;
}

int do_upload(bsam_hier h, const bsam_hier_desc *d) {
  int rc = validate(d);
  if (rc) return rc;
  cudaStream_t s = h->stream;
  h->nlev = d->nlev;
  h->root = d->root_idx;
  h->npatch = d->npatch;
  h->hpatches.assign(d->patches, d->patches + (size_t)d->npatch * PDN);
  h->hlevels.assign(d->levels, d->levels + (size_t)d->nlev * LDN);
  h->hs.assign(d->hs, d->hs + 2 * d->nlev);
  h->n_q = d->n_q;
  h->n_cells = d->n_cells;
  h->n_qc = d->n_qc;
  h->ninst = d->ninst > 1 ? d->ninst : 1;
  std::vector<int> pinst(d->npatch, 0);
  h->inst_root.assign(h->ninst, d->root_idx);
  if (h->ninst > 1) {
    pinst.assign(d->patch_inst, d->patch_inst + d->npatch);
    h->inst_root.assign(d->inst_root, d->inst_root + h->ninst);
  }
  int64_t asz = 0;
  for (int i = 0; i < h->ninst; ++i) {
    const int32_t *r1 = d->patches + (size_t)i * PDN;
    asz += (int64_t)r1[PD_MX] * r1[PD_MY] * r1[PD_MX] * r1[PD_MY];
  }
  if ((rc = h->Q.upload(d->Q, d->n_q, s)) || (rc = h->F.upload(d->F, d->n_cells, s)) ||
      (rc = h->FTrue.upload(d->FTrue, d->n_cells, s)) || (rc = h->CC.upload(d->CC, d->n_cells, s)) ||
      (rc = h->ID.upload(d->InvDiagS, d->n_cells, s)) || (rc = h->DeW.upload(d->DeW, d->n_dew, s)) ||
      (rc = h->DnS.upload(d->DnS, d->n_dns, s)) || (rc = h->QC.upload(d->QC, d->n_qc, s)) ||
      (rc = h->bcg.upload(d->bcg, d->n_bcg, s)) || (rc = h->cfd.upload(d->cfd, d->n_cfd, s)) ||
      (rc = h->pcoef.upload(d->pcoef, d->n_pcoef, s)) || (rc = h->win.upload(d->win, d->n_win, s)) ||
      (rc = h->fp.upload(d->fp, 2 * d->n_fp, s)) || (rc = h->ring.upload(d->ring, 2 * d->n_ring, s)) ||
      (rc = h->Ainv.upload(d->Ainv, (size_t)asz, s)) || (rc = h->bcRhs.upload(d->bcRhs, d->ncoarse, s)))
    return rc;
  // patches
  std::vector<PatchD> pd(d->npatch);
  for (int p = 0; p < d->npatch; ++p) {
    const int32_t *r = d->patches + (size_t)p * PDN;
    PatchD &q = pd[p];
    q.mx = r[PD_MX]; q.my = r[PD_MY]; q.par0 = r[PD_PAR0]; q.level = r[PD_LEVEL];
    q.q_off = r[PD_QOFF]; q.c_off = r[PD_COFF]; q.dew_off = r[PD_DEWOFF]; q.dns_off = r[PD_DNSOFF];
    q.qc_off = r[PD_QCOFF]; q.bcg_off = r[PD_BCGOFF]; q.cfd_off = r[PD_CFDOFF]; q.pc_off = r[PD_PCOFF];
    q.win_off = r[PD_WIN0]; q.fp_off = r[PD_FP0]; q.corr_off = r[PD_CORR0]; q.pe_off = 0;
    for (int sd = 0; sd < 4; ++sd) q.bc[sd] = r[PD_BCW + sd];
    q.inst = pinst[p];
    const int root = h->inst_root[q.inst];
    q.pflags = (q.level >= root ? 1 : 0) | (q.level >= std::max(2, root + 1) ? 2 : 0);
    q.ilo = r[PD_ILO];
    q.jlo = r[PD_JLO];
  }
  // plan
  Builder B{h, d};
  B.pe_off.assign(d->npatch, 0);
  B.pinst = pinst;
  h->lev.assign(d->nlev + 1, LevelPlan());
  std::vector<uint8_t> flags(d->covered, d->covered + d->n_cells);
  std::vector<int> ct_cell, ct_patch, ct_beg, ct_item, ct_j;
  for (int k = 1; k <= d->nlev; ++k) {
    LevelPlan &L = h->lev[k];
    const int32_t *lv = d->levels + (size_t)(k - 1) * LDN;
    L.k = k;
    L.p0 = lv[LD_P0];
    L.p1 = lv[LD_P1];
    L.hx = d->hs[2 * (k - 1)];
    L.hy = d->hs[2 * (k - 1) + 1];
    L.pow2 = is_pow2(L.hx * L.hx) && is_pow2(L.hy * L.hy);
    L.ncells = lv[LD_CELL1] - lv[LD_CELL0];
    L.col = B.make_decomp(L.p0, L.p1, 0);
    L.cell = B.make_decomp(L.p0, L.p1, 1);
    if (k > 1) L.coarse = B.make_decomp(L.p0, L.p1, 2);
    if (k > 1) {
      L.ring_off = B.P(L.p0)[PD_RING0];
      L.ring_n = B.P(L.p1 - 1)[PD_RING1] - L.ring_off;
    }
    if ((rc = B.ghosts(k, L))) return rc;
    // flux corrections of this level's patches, gathered per target cell
    if (k > 1) {
      struct It { int cell, item, j; };
      std::vector<It> items;
      for (int p = L.p0; p < L.p1; ++p) {
        const int32_t *r = B.P(p);
        const int cmx = r[PD_MX] / 2, cmy = r[PD_MY] / 2;
        int o = r[PD_CORR0];
        for (int f = 0; f < 4; ++f) {
          const int nn = f < 2 ? cmy : cmx;
          for (int j = 0; j < nn; ++j) {
            const int t = d->corr[o + j];
            if (t >= 0) items.push_back({t, ((p - L.p0) << 2) | f, j});
          }
          o += nn;
        }
      }
      std::stable_sort(items.begin(), items.end(), [](const It &a, const It &b) { return a.cell < b.cell; });
      const LevelPlan &Lc = h->lev[k - 1];
      L.ct_off = (int)ct_cell.size();
      for (size_t i = 0; i < items.size();) {
        size_t e = i;
        while (e < items.size() && items[e].cell == items[i].cell) ++e;
        const int cell = items[i].cell;
        // owning patch of the target in level k-1
        int q = -1;
        for (int pp = Lc.p0; pp < Lc.p1; ++pp) {
          const int32_t *rq = B.P(pp);
          if (cell >= rq[PD_COFF] && cell < rq[PD_COFF] + rq[PD_MX] * rq[PD_MY]) { q = pp - Lc.p0; break; }
        }
        if (q < 0) return fail(BSAM_ERR_ARG, "correction target is not a cell of the parent level");
        ct_cell.push_back(cell);
        ct_patch.push_back(q);
        ct_beg.push_back((int)ct_item.size());
        for (size_t t = i; t < e; ++t) {
          ct_item.push_back(items[t].item);
          ct_j.push_back(items[t].j);
        }
        flags[cell] |= 2;
        i = e;
      }
      L.ct_n = (int)ct_cell.size() - L.ct_off;
      // sentinel row so that tbeg[t + 1] exists for the level's last target
      ct_cell.push_back(0);
      ct_patch.push_back(0);
      ct_beg.push_back((int)ct_item.size());
    }
  }
  for (int p = 0; p < d->npatch; ++p) pd[p].pe_off = B.pe_off[p];
  if ((rc = h->patches.upload(pd.data(), pd.size(), s))) return rc;
  if (B.perim.empty()) B.perim.push_back(Rule{-1, 0, 0, 0, 0, 0, 0, 0});
  std::vector<RelaxChunkD> dchunks(B.chunks.size());
  for (size_t i = 0; i < B.chunks.size(); ++i) {
    const RelaxChunk &c = B.chunks[i];
    int fl = (c.par0 & 1) << 8;
    for (int sd = 0; sd < 4; ++sd) fl |= c.bc[sd] << (2 * sd);   // codes 0..2, checked above
    dchunks[i] = RelaxChunkD{c.q_off, c.c_off, c.bcg_off, c.pe_off, c.mx, c.my, c.s0, c.n, c.inst, fl, 0, 0};
  }
  if ((rc = h->perim.upload(B.perim.data(), B.perim.size(), s)) ||
      (rc = h->rchunks.upload(dchunks.data(), dchunks.size(), s)))
    return rc;
  // frozen-chunk flags of a batch: each instance's chunks form one range per
  // level (instances stored one after another within a level, checked in
  // validate)
  h->act_mode = h->ninst > 1 ? kActChunk : kActNone;
  if (h->ninst > 1) {
    const int nl = d->nlev;
    std::vector<int> cr((size_t)h->ninst * nl * 2, 0), cnt((size_t)h->ninst * nl, 0);
    for (int k = 1; k <= nl; ++k) {
      const LevelPlan &L = h->lev[k];
      for (int c = L.rc_off; c < L.rc_off + L.rc_n; ++c) {
        const size_t e = (size_t)B.chunks[c].inst * nl + (k - 1);
        if (!cnt[e]) cr[2 * e] = c;
        cr[2 * e + 1] = c + 1;
        ++cnt[e];
      }
    }
    for (size_t e = 0; e < cnt.size(); ++e)
      if (cnt[e] && cnt[e] != cr[2 * e + 1] - cr[2 * e])
        return fail(BSAM_ERR_ARG, "batch chunks of an instance are not one range per level");
    {
      if ((rc = h->crange.upload(cr.data(), cr.size(), s)) || (rc = h->cact.alloc(std::max<size_t>(B.chunks.size(), 1))))
        return rc;
      CK(cudaMemsetAsync(h->cact.p, 1, h->cact.n, s));
    }
  }
  // smoother operands, the face coefficients exactly scaled by 1/h^2 on
  // power-of-two levels, packed on the device
  {
    if ((rc = h->pchunks.upload(B.chunks.data(), B.chunks.size(), s)) || (rc = build_relax_pack(h))) return rc;
    h->relax_n[0].assign(d->nlev + 1, 1);
    h->relax_n[1].assign(d->nlev + 1, 1);
  }
  // residual plan: warp tasks, slots in instance order, level by level
  constexpr int kTask = 32 * kResLane;
  // (main cells, then the level's correction targets), then the QC refresh
  // tasks of the levels above each instance's root
  std::vector<ResTask> tasks;
  std::vector<SlotRange> ranges;
  std::vector<InstRes> ir(h->ninst);
  h->inst_visible.assign(h->ninst, 0);
  int ns = 0;
  for (int i = 0; i < h->ninst; ++i) {
    ir[i].range0 = (int)ranges.size();
    for (int k = h->inst_root[i]; k <= d->nlev; ++k) {
      const LevelPlan &L = h->lev[k];
      const int s0 = ns;
      for (int p = L.p0; p < L.p1; ++p) {
        if (pinst[p] != i) continue;
        const int32_t *r = B.P(p);
        const int n = r[PD_MX] * r[PD_MY];
        for (int c = 0; c < n; ++c) h->inst_visible[i] += (d->covered[r[PD_COFF] + c] == 0);
        for (int b0 = 0; b0 < n; b0 += kTask) tasks.push_back(ResTask{0, k, p, b0, std::min(kTask, n - b0), ns++, i, 0});
      }
      if (k < d->nlev) {
        const LevelPlan &Lf = h->lev[k + 1];
        // targets of this instance: a contiguous run (cells are ordered by patch)
        int t0 = -1, t1 = -1;
        for (int t = 0; t < Lf.ct_n; ++t)
          if (pinst[L.p0 + ct_patch[Lf.ct_off + t]] == i) {
            if (t0 < 0) t0 = t;
            t1 = t + 1;
          }
        for (int t = t0; t0 >= 0 && t < t1; t += kTask)
          tasks.push_back(ResTask{1, k, 0, t, std::min(kTask, t1 - t), ns++, i, 0});
      }
      ranges.push_back(SlotRange{s0, ns, L.hx * L.hy});
    }
    ir[i].range1 = (int)ranges.size();
    ir[i].max_vcycles = h->opts.max_vcycles;
    ir[i].pad = 0;
    ir[i].rel_tol = h->opts.rel_tol;
    ir[i].ncell = (double)h->inst_visible[i];
  }
  for (int k = 2; k <= d->nlev; ++k) {
    const LevelPlan &L = h->lev[k];
    for (int p = L.p0; p < L.p1; ++p) {
      const int32_t *r = B.P(p);
      const int root = h->inst_root[pinst[p]];
      if (k < std::max(2, root + 1)) continue;
      for (int t = r[PD_RING0]; t < r[PD_RING1]; t += kTask)
        tasks.push_back(ResTask{2, k, t, 0, std::min(kTask, r[PD_RING1] - t), 0, pinst[p], 0});
      const int nc = (r[PD_MX] / 2) * (r[PD_MY] / 2);
      for (int b0 = 0; b0 < nc; b0 += kTask) tasks.push_back(ResTask{3, k, p, b0, std::min(kTask, nc - b0), 0, pinst[p], 0});
    }
  }
  h->nrtasks = (int)tasks.size();
  h->nslots = std::max(ns, 1);
  // the instance's targets must be one run per level
  for (int k = 2; k <= d->nlev; ++k) {
    const LevelPlan &L = h->lev[k];
    for (int t = 1; t < L.ct_n; ++t)
      if (pinst[h->lev[k - 1].p0 + ct_patch[L.ct_off + t]] < pinst[h->lev[k - 1].p0 + ct_patch[L.ct_off + t - 1]])
        return fail(BSAM_ERR_ARG, "batch patches of a level must be grouped by instance");
  }
  // coarsest: one dense inverse block per instance
  std::vector<CoarsestD> cds(h->ninst);
  {
    long long ao = 0, ro = 0;
    h->coarse_max_rows = 0;
    for (int i = 0; i < h->ninst; ++i) {
      const int32_t *r1 = B.P(i);
      CoarsestD &c = cds[i];
      c.c_off = r1[PD_COFF];
      c.q_off = r1[PD_QOFF];
      c.n1 = r1[PD_MX];
      c.N = r1[PD_MX] * r1[PD_MY];
      c.inst = i;
      c.pad = 0;
      c.ainv_off = ao;
      c.rhs_off = ro;
      ao += (long long)c.N * c.N;
      ro += c.N;
      h->coarse_max_rows = std::max(h->coarse_max_rows, c.N);
    }
    h->ncoarse_patches = h->ninst;
    h->ncoarse_total = ro;
  }
  h->all_cells = B.make_decomp(0, d->npatch, 1);
  h->below_top = B.make_decomp(0, h->lev[d->nlev].p0, 1);
  // a level whose Q range holds only its own patches (the FP32 cycle's
  // zero-parent fill takes every operand outside the range for a parent cell)
  for (int k = 1; k <= d->nlev; ++k) {
    LevelPlan &L = h->lev[k];
    bool own = true;
    for (int p = 0; p < d->npatch && own; ++p) {
      if (p >= L.p0 && p < L.p1) continue;
      const int32_t *r = B.P(p);
      const int64_t a = r[PD_QOFF], b = a + (int64_t)(r[PD_MX] + 2) * (r[PD_MY] + 2);
      own = b <= L.q_lo || a >= L.q_hi;
    }
    L.range_own = own;
  }
  // k_restrict_update skips the covered cells of the levels below the
  // finest: exact where those are exactly the cells some restriction writes
  {
    std::vector<uint8_t> target((size_t)d->n_q, 0);
    for (int64_t i = 0; i < d->n_fp; ++i) target[(size_t)d->fp[2 * i]] = 1;
    bool same = d->nlev >= 2;
    for (int p = 0; p < h->lev[d->nlev].p0 && same; ++p) {
      const int32_t *r = B.P(p);
      const int mx = r[PD_MX], my = r[PD_MY];
      for (int lj = 0; lj < my && same; ++lj)
        for (int lx = 0; lx < mx; ++lx) {
          const bool cov = d->covered[r[PD_COFF] + lx + lj * mx] != 0;
          const bool tgt = target[(size_t)r[PD_QOFF] + (lx + 1) + (lj + 1) * (mx + 2)] != 0;
          if (cov != tgt) { same = false; break; }
        }
    }
    h->update_fold = same;
  }
  std::vector<int> rinst(std::max<int64_t>(d->n_ring, 1), 0);
  for (int p = 0; p < d->npatch; ++p)
    for (int t = B.P(p)[PD_RING0]; t < B.P(p)[PD_RING1]; ++t) rinst[t] = pinst[p];
  h->hir = ir;
  h->hist_stride = h->opts.max_vcycles + 1;
  std::vector<int> inlev(h->ninst, 0);
  for (int p = 0; p < d->npatch; ++p) inlev[pinst[p]] = std::max(inlev[pinst[p]], (int)B.P(p)[PD_LEVEL]);
  // fused-fill operands: for the ghost items of each level k-1 (k >= 2),
  // the cells of level k-1 that the restriction from level k overwrites,
  // with the four fine cells they are restricted from (ebTransfer.m:10-33)
  {
    std::vector<int> aa(B.ga), ab(B.gb), ac(B.gc);
    std::vector<int2> rt;
    for (int k = 2; k <= d->nlev; ++k) {
      const LevelPlan &L = h->lev[k], &Lc = h->lev[k - 1];
      if (!Lc.g1_n) continue;
      std::unordered_map<int, int> cov;   // parent Q index -> entry of rt
      for (int p = L.p0; p < L.p1; ++p) {
        const int32_t *r = B.P(p);
        const int mx = r[PD_MX], cmx = mx / 2, cmy = r[PD_MY] / 2, ldq = mx + 2;
        for (int sidx = 0; sidx < cmx * cmy; ++sidx) {
          const int cj = sidx / cmx, ci = sidx - cj * cmx;
          const int dst = d->fp[2 * (r[PD_FP0] + sidx)];
          cov[dst] = (int)rt.size();
          rt.push_back(make_int2(r[PD_QOFF] + (2 * ci + 1) + (2 * cj + 1) * ldq, ldq));
        }
      }
      auto code = [&](int q) {
        auto it = cov.find(q);
        return it == cov.end() ? q : -1 - it->second;
      };
      for (int i = Lc.g1_off; i < Lc.g1_off + Lc.g1_n; ++i) {
        const int8_t t = B.gt[i];
        if (t == G_RING) continue;               // source in the level below: never restricted
        if (t == G_PHYS_CORNER) { ac[i] = code(B.gc[i]); continue; }   // a, b: rule indices
        aa[i] = code(B.ga[i]);
        if (t == G_QIF || t == G_QIF_END || t == G_LIF || t == G_DIRICHLET) ab[i] = code(B.gb[i]);
        if (t == G_QIF || t == G_QIF_END || t == G_LIF || t == G_LIF_CORNER) ac[i] = code(B.gc[i]);
      }
      // level k's own fill in the same launch (launch_restrict_fill with
      // fill_k): allowed when no rule of it reads a cell the restriction or
      // the parent's fill writes and the parent's fill reads no ghost cell of
      // level k.  Its ring items read parent cells, which the restriction
      // overwrites where a sibling patch covers them: after the
      // pre-smoothing they are left out (the coarse load refreshes every
      // ring cell of the level before anything reads one); before the
      // fill-down they must run, so they must read no such cell.
      std::unordered_map<int, int> pw, gw;   // Q cells the parent's / level k's fill writes
      for (int i = Lc.g1_off; i < Lc.g1_off + Lc.g1_n; ++i)
        if (B.gt[i] != G_RING) pw[B.gdst[i]] = i;
      for (int i = L.g1_off; i < L.g1_off + L.g1_n; ++i)
        if (B.gt[i] != G_RING) gw[B.gdst[i]] = i;
      std::vector<int> rd;
      bool ok = true, ring_ok = true, rpg = false;
      for (int i = L.g1_off; i < L.g1_off + L.g1_n; ++i) {
        rd.clear();
        ghost_reads(B, i, rd);
        for (int q : rd) {
          const bool g = pw.count(q) > 0, hit = g || cov.count(q);
          rpg |= g;
          if (B.gt[i] == G_RING) ring_ok &= !hit;
          else ok &= !hit;
        }
      }
      h->lev[k].reads_pg = rpg;
      for (int i = Lc.g1_off; i < Lc.g1_off + Lc.g1_n && ok; ++i) {
        rd.clear();
        ghost_reads(B, i, rd);
        for (int q : rd) ok &= !gw.count(q);
      }
      h->lev[k].fuse_pre = ok;
      h->lev[k].fuse_top = ok && ring_ok;
    }
    // windows: parent ghost cells -> the parent level's item filling them
    std::vector<int> walt(d->win, d->win + d->n_win);
    for (int k = 2; k <= d->nlev; ++k) {
      const LevelPlan &L = h->lev[k], &Lc = h->lev[k - 1];
      std::unordered_map<int, int> gh;     // parent Q ghost cell -> ghost item
      for (int i = Lc.g1_off; i < Lc.g1_off + Lc.g1_n; ++i)
        if (B.gt[i] != G_RING) gh[B.gdst[i]] = i;
      for (int p = L.p0; p < L.p1; ++p) {
        const int32_t *r = B.P(p);
        const int nw = (r[PD_MX] / 2 + 2) * (r[PD_MY] / 2 + 2);
        for (int w = r[PD_WIN0]; w < r[PD_WIN0] + nw; ++w) {
          auto it = gh.find(d->win[w]);
          if (it != gh.end()) walt[w] = -1 - it->second;
        }
      }
    }
    if (walt.empty()) walt.push_back(0);
    if ((rc = h->win_alt.upload(walt.data(), walt.size(), s))) return rc;
    if (rt.empty()) rt.push_back(make_int2(0, 0));
    if ((rc = h->ga_a.upload(aa.data(), aa.size(), s)) || (rc = h->ga_b.upload(ab.data(), ab.size(), s)) ||
        (rc = h->ga_c.upload(ac.data(), ac.size(), s)) || (rc = h->ga_rt.upload(rt.data(), rt.size(), s)))
      return rc;
  }
  if ((rc = h->g_inst.upload(B.gi.data(), B.gi.size(), s)) || (rc = h->ring_inst.upload(rinst.data(), rinst.size(), s)) ||
      (rc = h->inst_nlev.upload(inlev.data(), inlev.size(), s)))
    return rc;
  if ((rc = h->flags.upload(flags.data(), flags.size(), s)) || (rc = h->ints.upload(B.ints.data(), B.ints.size(), s)) ||
      (rc = h->g_type.upload(B.gt.data(), B.gt.size(), s)) || (rc = h->g_dst.upload(B.gdst.data(), B.gdst.size(), s)) ||
      (rc = h->g_a.upload(B.ga.data(), B.ga.size(), s)) || (rc = h->g_b.upload(B.gb.data(), B.gb.size(), s)) ||
      (rc = h->g_c.upload(B.gc.data(), B.gc.size(), s)) || (rc = h->g_d.upload(B.gd.data(), B.gd.size(), s)) ||
      (rc = h->g_e.upload(B.ge.data(), B.ge.size(), s)) || (rc = h->ct_cell.upload(ct_cell.data(), ct_cell.size(), s)) ||
      (rc = h->ct_patch.upload(ct_patch.data(), ct_patch.size(), s)) ||
      (rc = h->ct_beg.upload(ct_beg.data(), ct_beg.size(), s)) ||
      (rc = h->ct_item.upload(ct_item.data(), ct_item.size(), s)) || (rc = h->ct_j.upload(ct_j.data(), ct_j.size(), s)) ||
      (rc = h->rtasks.upload(tasks.data(), tasks.size(), s)) || (rc = h->sranges.upload(ranges.data(), ranges.size(), s)) ||
      (rc = h->instres.upload(ir.data(), ir.size(), s)) || (rc = h->coarsest.upload(cds.data(), cds.size(), s)) ||
      (rc = h->slots.alloc(3 * (size_t)h->nslots)) || (rc = h->acc.alloc(h->ninst)) ||
      (rc = h->iters.alloc(h->ninst)) ||
      (rc = h->hist.alloc((size_t)h->ninst * h->hist_stride)))
    return rc;
  // per-level descriptors for the residual kernel
  {
    std::vector<LevelX> X(d->nlev + 2);
    std::memset(X.data(), 0, sizeof(LevelX) * X.size());
    for (int k = 1; k <= d->nlev; ++k) {
      LevelPlan &L = h->lev[k];
      X[k].L = leveld(h, k);
      X[k].C = corr_csr(h, L);
      X[k].ct_n = L.ct_n;
      X[k].pad = 0;
    }
    if ((rc = h->levelx.upload(X.data(), X.size(), s))) return rc;
  }
  CK(cudaMemsetAsync(h->acc.p, 0, sizeof(ResAcc) * h->ninst, s));
  CK(cudaMemsetAsync(h->iters.p, 0, sizeof(int) * h->ninst, s));
  CK(cudaMemsetAsync(h->hist.p, 0, sizeof(double) * h->hist.n, s));
  {
    // every instance starts active: eager operations (ghost fills, prolong,
    // fill-down) apply to all of them
    std::vector<int> one(h->ninst, 1);
    if ((rc = h->active.upload(one.data(), one.size(), s)) || (rc = h->ones.upload(one.data(), one.size(), s))) return rc;
  }
  // partial sums for composite sums
  int np = 0;
  for (int k = 1; k <= d->nlev; ++k) np += h->lev[k].cell.nblocks;
  h->npartials = np;
  if ((rc = h->partials.alloc((size_t)4 * std::max(np, 1)))) return rc;
  h->acc_host = new ResAcc[h->ninst]();
  h->active_host = new int[h->ninst]();
  CK(cudaStreamSynchronize(s));
  return BSAM_OK;
}

void release(bsam_hier h) {
  drop_graph(h);
  for (DBuf<double> *b : {&h->Q, &h->F, &h->FTrue, &h->QC, &h->CC, &h->ID, &h->DeW, &h->DnS, &h->bcg, &h->cfd,
                          &h->pcoef, &h->Ainv, &h->bcRhs, &h->slots, &h->partials, &h->hist, &h->saveQ, &h->saveQC, &h->rpack, &h->Uo, &h->Uoo, &h->fsrc,
                          &h->saveF})
    b->release();
  for (DBuf<float> *b : {&h->E, &h->F32, &h->QC32, &h->DeW32, &h->DnS32, &h->CC32, &h->ID32, &h->pcoef32, &h->cfd32,
                         &h->bcg32, &h->rpack32})
    b->release();
  for (DBuf<int> *b : {&h->win, &h->fp, &h->ring, &h->ints, &h->ct_cell, &h->ct_patch, &h->ct_beg, &h->ct_item,
                       &h->ct_j, &h->active, &h->iters, &h->ones, &h->g_inst, &h->ring_inst, &h->inst_nlev, &h->g_dst, &h->g_a, &h->g_b, &h->g_c, &h->g_d, &h->g_e,
                       &h->ga_a, &h->ga_b, &h->ga_c, &h->win_alt})
    b->release();
  h->flags.release(); h->g_type.release(); h->patches.release(); h->acc.release(); h->perim.release();
  h->rchunks.release(); h->pchunks.release(); h->cact.release(); h->crange.release(); h->levelx.release(); h->rtasks.release(); h->instres.release(); h->sranges.release();
  h->coarsest.release();
  h->ga_rt.release();
  delete[] h->acc_host;
  delete[] h->active_host;
  h->acc_host = nullptr;
  h->active_host = nullptr;
}

int check_opts(const bsam_solve_opts *o) {
  if (!o || o->npre < 0 || o->npost < 0 || o->max_vcycles < 0 || !(o->rel_tol >= 0) || !(o->omega > 0) ||
      (o->ghost_interp != 0 && o->ghost_interp != 1) || (o->precision != 0 && o->precision != 1))
    return fail(BSAM_ERR_ARG, "invalid solve options");
  return BSAM_OK;
}

int set_device(bsam_hier h) {
  CK(cudaSetDevice(h->ctx->device));
  g_stream = h->stream;
  return BSAM_OK;
}

}  // namespace

// ===========================================================================
extern "C" {

const char *bsam_last_error(void) { return g_err.c_str(); }

int bsam_ctx_create(int device, bsam_ctx *out) {
  if (!out) return fail(BSAM_ERR_ARG, "null output");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return fail(BSAM_ERR_NODEV, "no CUDA device available");
  if (device < 0 || device >= n) return fail(BSAM_ERR_ARG, "device ordinal out of range");
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, device));
  if (prop.major != 10 || prop.minor != 3)
    return fail(BSAM_ERR_NODEV, std::string("libbsam_dev is built for sm_103a; device is ") + prop.name);
  CK(cudaSetDevice(device));
  bsam_ctx c = new bsam_ctx_s;
  c->device = device;
  cudaError_t se = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (se != cudaSuccess) {
    delete c;
    return cuda_fail(se, "cudaStreamCreate");
  }
  // this process's device buffers come from the device's default memory
  // pool in stream order; freed blocks stay in the pool for the next
  // hierarchy instead of being released to the CUDA driver at every synchronisation
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  cudaGetLastError();
  *out = c;
  return BSAM_OK;
}

int bsam_device_memory(int device, int64_t *free_bytes, int64_t *total_bytes) {
  if (!free_bytes || !total_bytes) return fail(BSAM_ERR_ARG, "null output");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
    return fail(BSAM_ERR_NODEV, "no such CUDA device");
  CK(cudaSetDevice(device));
  size_t f = 0, t = 0;
  CK(cudaMemGetInfo(&f, &t));
  *free_bytes = (int64_t)f;
  *total_bytes = (int64_t)t;
  return BSAM_OK;
}

int bsam_fp64_rate(bsam_ctx ctx, double *gops) {
  if (!ctx || !gops) return fail(BSAM_ERR_ARG, "null argument");
  CK(cudaSetDevice(ctx->device));
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const int blocks = sms * 8, iters = 1024;
  double *out = nullptr;
  CK(cudaMallocAsync((void **)&out, sizeof(double) * blocks * kBlock, ctx->stream));
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  for (int r = 0; r < 4; ++r) {
    cudaEventRecord(a, ctx->stream);
    k_fp64_rate<<<blocks, kBlock, 0, ctx->stream>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(b, ctx->stream);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (r > 0) best = std::min(best, ms);     // the first is a warm-up
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  const cudaError_t e = cudaGetLastError();
  cudaFreeAsync(out, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(e, "bsam_fp64_rate");
  *gops = (double)kFp64RateOps * iters * blocks * kBlock / (best * 1e-3) / 1e9;
  return BSAM_OK;
}

// drops one reference to the context (its creator's, or a hierarchy's) and
// destroys it with the last one
static void ctx_unref(bsam_ctx ctx) {
  {
    std::lock_guard<std::mutex> lk(ctx->ref_mu);
    if (--ctx->refs > 0) return;
  }
  cudaSetDevice(ctx->device);
  if (ctx->scratch) cudaFreeAsync(ctx->scratch, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int bsam_ctx_destroy(bsam_ctx ctx) {
  if (!ctx) return BSAM_OK;
  ctx_unref(ctx);
  return BSAM_OK;
}

int bsam_hier_upload(bsam_ctx ctx, const bsam_hier_desc *desc, const bsam_solve_opts *opts, bsam_hier *out) {
  if (!ctx || !out) return fail(BSAM_ERR_ARG, "null argument");
  int rc = check_opts(opts);
  if (rc) return rc;
  bsam_hier h = new bsam_hier_s;
  h->ctx = ctx;
  h->stream = ctx->stream;
  h->opts = *opts;
  if ((rc = set_device(h)) || (rc = do_upload(h, desc))) {
    release(h);
    delete h;
    return rc;
  }
  {
    std::lock_guard<std::mutex> lk(ctx->ref_mu);
    ++ctx->refs;
  }
  *out = h;
  return BSAM_OK;
}

int bsam_hier_free(bsam_hier h) {
  if (!h) return BSAM_OK;
  set_device(h);
  cudaStreamSynchronize(h->stream);
  release(h);
  bsam_ctx ctx = h->ctx;
  delete h;
  ctx_unref(ctx);
  return BSAM_OK;
}

int bsam_set_opts(bsam_hier h, const bsam_solve_opts *opts) {
  if (!h) return fail(BSAM_ERR_ARG, "null hierarchy");
  int rc = check_opts(opts);
  if (rc) return rc;
  const bool replan = opts->ghost_interp != h->opts.ghost_interp;
  if (replan) return fail(BSAM_ERR_STATE, "GhostInterp is fixed at upload; upload the hierarchy again");
  h->opts = *opts;
  drop_graph(h);
  rc = set_device(h);
  if (rc) return rc;
  return apply_opts(h);
}

static int ensure_history(bsam_hier h) {
  int rc;
  if (!h->Uo.p) {
    if ((rc = h->Uo.alloc(h->n_cells)) || (rc = h->Uoo.alloc(h->n_cells))) return rc;
    CK(cudaMemsetAsync(h->Uo.p, 0, sizeof(double) * h->n_cells, h->stream));
    CK(cudaMemsetAsync(h->Uoo.p, 0, sizeof(double) * h->n_cells, h->stream));
  }
  return BSAM_OK;
}

static DBuf<double> *field_buf(bsam_hier h, int which) {
  switch (which) {
    case BSAM_FIELD_Q: return &h->Q;
    case BSAM_FIELD_F: return &h->F;
    case BSAM_FIELD_FTRUE: return &h->FTrue;
    case BSAM_FIELD_QC: return &h->QC;
    case BSAM_FIELD_CC: return &h->CC;
    case BSAM_FIELD_INVDIAG: return &h->ID;
    case BSAM_FIELD_DEW: return &h->DeW;
    case BSAM_FIELD_DNS: return &h->DnS;
    case BSAM_FIELD_PCOEF: return &h->pcoef;
    case BSAM_FIELD_CFD: return &h->cfd;
    case BSAM_FIELD_BCG: return &h->bcg;
    case BSAM_FIELD_AINV: return &h->Ainv;
    case BSAM_FIELD_BCRHS: return &h->bcRhs;
    case BSAM_FIELD_UO: return ensure_history(h) ? nullptr : &h->Uo;
    case BSAM_FIELD_UOO: return ensure_history(h) ? nullptr : &h->Uoo;
    default: return nullptr;
  }
}

// the smoother's packed operands after an update of DeW, DnS or InvDiagS

int bsam_set_field(bsam_hier h, int which, const double *host, int64_t n) {
  if (!h || !host) return fail(BSAM_ERR_ARG, "null argument");
  int rc = set_device(h);
  if (rc) return rc;
  DBuf<double> *b = field_buf(h, which);
  if (!b) return fail(BSAM_ERR_ARG, "unknown field");
  if ((size_t)n != b->n) return fail(BSAM_ERR_ARG, "field length mismatch");
    if (n) CK(cudaMemcpyAsync(b->p, host, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (which == BSAM_FIELD_DEW || which == BSAM_FIELD_DNS || which == BSAM_FIELD_INVDIAG) {
    if ((rc = build_relax_pack(h))) return rc;
  }
  if (which >= BSAM_FIELD_CC && which <= BSAM_FIELD_BCRHS) h->f32_dirty = true;
  return BSAM_OK;
}

int bsam_get_field(bsam_hier h, int which, double *host, int64_t n) {
  if (!h || !host) return fail(BSAM_ERR_ARG, "null argument");
  int rc = set_device(h);
  if (rc) return rc;
  DBuf<double> *b = field_buf(h, which);
  if (!b) return fail(BSAM_ERR_ARG, "unknown field");
  if ((size_t)n != b->n) return fail(BSAM_ERR_ARG, "field length mismatch");
  if (n) CK(cudaMemcpyAsync(host, b->p, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return BSAM_OK;
}

int bsam_fill_ghosts(bsam_hier h, int level) {
  if (!h || level < 1 || level > h->nlev) return fail(BSAM_ERR_ARG, "level out of range");
  int rc = set_device(h);
  if (rc) return rc;
  launch_fill(h, level);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->stream));
  return BSAM_OK;
}

int bsam_prolong_level(bsam_hier h, int level) {
  if (!h || level < 2 || level > h->nlev) return fail(BSAM_ERR_ARG, "level out of range");
  int rc = set_device(h);
  if (rc) return rc;
  launch_prolong(h, level, 0);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->stream));
  return BSAM_OK;
}

int bsam_filldown(bsam_hier h) {
  if (!h) return fail(BSAM_ERR_ARG, "null hierarchy");
  int rc = set_device(h);
  if (rc) return rc;
  launch_filldown(h);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->stream));
  return BSAM_OK;
}

int bsam_comp_residual(bsam_hier h, double out[5]) {
  if (!h || !out) return fail(BSAM_ERR_ARG, "null argument");
  int rc = set_device(h);
  if (rc) return rc;
  launch_residual(h, 2);
  CK(cudaGetLastError());
  return read_residual(h, out);
}

int bsam_setup_levels(bsam_hier h) {
  if (!h) return fail(BSAM_ERR_ARG, "null hierarchy");
  int rc = set_device(h);
  if (rc) return rc;
  std::vector<int> mask(h->ninst);
  for (int k = 1; k <= h->nlev; ++k) {
    bool any = false;
    for (int i = 0; i < h->ninst; ++i) {
      mask[i] = k > h->inst_root[i] ? 1 : 0;
      any = any || mask[i];
    }
    if (any && k > 1) {
      // mask staged through the pinned per-instance buffer, stream-ordered
      CK(cudaStreamSynchronize(h->stream));
      std::copy(mask.begin(), mask.end(), h->active_host);
      CK(cudaMemcpyAsync(h->active.p, h->active_host, sizeof(int) * h->ninst, cudaMemcpyHostToDevice, h->stream));
      launch_prolong(h, k, 0);
      CK(cudaMemcpyAsync(h->active.p, h->ones.p, sizeof(int) * h->ninst, cudaMemcpyDeviceToDevice, h->stream));
    }
    launch_fill(h, k);
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->stream));
  return BSAM_OK;
}

int bsam_parabolic_rhs(bsam_hier h, int scheme, double dt, const double *f, int64_t n) {
  if (!h) return fail(BSAM_ERR_ARG, "null hierarchy");
  if ((scheme != 0 && scheme != 1) || !(dt > 0)) return fail(BSAM_ERR_ARG, "bad scheme or time step");
  if (f && n != h->n_cells) return fail(BSAM_ERR_ARG, "source length mismatch");
  int rc = set_device(h);
  if (rc || (rc = ensure_history(h))) return rc;
  if (f) {
    if (!h->fsrc.p && (rc = h->fsrc.alloc(h->n_cells))) return rc;
    CK(cudaMemcpyAsync(h->fsrc.p, f, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
  }
  Decomp D = decomp(h, h->all_cells);
  launch_k(h, k_prhs, D.nblocks, kBlock, D, (const PatchD *)h->patches.p, h->FTrue.p,
           (const double *)(f ? h->fsrc.p : nullptr), (const double *)h->Uo.p, (const double *)h->Uoo.p, dt, scheme);
  h->launch_count++;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->stream));
  return BSAM_OK;
}

int bsam_history_push(bsam_hier h) {
  if (!h) return fail(BSAM_ERR_ARG, "null hierarchy");
  int rc = set_device(h);
  if (rc || (rc = ensure_history(h))) return rc;
  Decomp D = decomp(h, h->all_cells);
  launch_k(h, k_history, D.nblocks, kBlock, D, (const PatchD *)h->patches.p, (const double *)h->Q.p, h->Uo.p,
           h->Uoo.p, 1);
  h->launch_count++;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->stream));
  return BSAM_OK;
}

int bsam_history_transfer(bsam_hier hn, bsam_hier hold, const int32_t *src_old, int64_t n, int has_uoo) {
  if (!hn || !hold || !src_old) return fail(BSAM_ERR_ARG, "null argument");
  if (hn == hold) return fail(BSAM_ERR_ARG, "the new and the old hierarchy must differ");
  if (n != hn->n_cells) return fail(BSAM_ERR_ARG, "source table length mismatch");
  if (hn->ctx->device != hold->ctx->device) return fail(BSAM_ERR_ARG, "hierarchies on different devices");
  // every cell at or above the root reads a valid old cell or derives from
  // its parent; the root has no parent, so every root cell has an old source
  const int root = std::max(hn->root, 1);
  for (int k = root; k <= hn->nlev; ++k) {
    const int64_t c0 = hn->hlevels[(size_t)(k - 1) * LDN + LD_CELL0], c1 = hn->hlevels[(size_t)(k - 1) * LDN + LD_CELL1];
    for (int64_t c = c0; c < c1; ++c) {
      if (src_old[c] >= hold->n_cells) return fail(BSAM_ERR_ARG, "source cell beyond the old hierarchy");
      if (src_old[c] < -1 || (k == root && src_old[c] < 0))
        return fail(BSAM_ERR_ARG, "root cell without an old source");
    }
  }
  int rc = set_device(hold);
  if (rc || (rc = ensure_history(hold))) return rc;
  CK(cudaStreamSynchronize(hold->stream));   // the old history is complete
  if ((rc = set_device(hn)) || (rc = ensure_history(hn))) return rc;
  DBuf<int> src;
  if ((rc = src.upload(src_old, (size_t)n, hn->stream))) return rc;
  if (has_uoo) {
    for (int k = root; k <= hn->nlev; ++k) {
      const LevelPlan &L = hn->lev[k];
      Decomp D = decomp(hn, L.cell);
      launch_k(hn, k_uoo_transfer, D.nblocks, kBlock, leveld(hn, k), D, (const int *)hn->fp.p, (const int *)src.p,
               (const double *)hold->Uoo.p, hn->Uoo.p);
      hn->launch_count++;
    }
  }
  Decomp D = decomp(hn, hn->all_cells);
  launch_k(hn, k_history, D.nblocks, kBlock, D, (const PatchD *)hn->patches.p, (const double *)hn->Q.p, hn->Uo.p,
           hn->Uoo.p, 0);
  hn->launch_count++;
  src.release();
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(hn->stream));
  return BSAM_OK;
}

int bsam_tag_level(bsam_hier h, int level, int indicator, double threshold, int buffer, int n0, int n1,
                   uint8_t *mask) {
  if (!h || !mask) return fail(BSAM_ERR_ARG, "null argument");
  if (level < 1 || level > h->nlev || (level == 1 && indicator == 1)) return fail(BSAM_ERR_ARG, "level out of range");
  if (indicator != 0 && indicator != 1) return fail(BSAM_ERR_ARG, "unknown indicator");
  if (h->ninst > 1) return fail(BSAM_ERR_STATE, "tagging runs on a single hierarchy, not a batch");
  if (n0 < 1 || n1 < 1 || buffer < 0) return fail(BSAM_ERR_ARG, "bad tag grid");
  const LevelPlan &L = h->lev[level];
  for (int p = L.p0; p < L.p1; ++p) {
    const int32_t *r = h->hpatches.data() + (size_t)p * PDN;
    if (r[PD_ILO] < 1 || r[PD_IHI] > n0 || r[PD_JLO] < 1 || r[PD_JHI] > n1)
      return fail(BSAM_ERR_ARG, "patch box outside the tag grid");
  }
  int rc = set_device(h);
  if (rc) return rc;
  const size_t n = (size_t)n0 * n1;
  uint8_t *buf = nullptr;
  CK(cudaMallocAsync((void **)&buf, 3 * n, h->stream));
  uint8_t *T = buf, *cover = buf + n, *out = buf + 2 * n;
  cudaError_t e = cudaMemsetAsync(buf, 0, 2 * n, h->stream);
  if (e == cudaSuccess) {
    if (indicator == 0) {
      Decomp D = decomp(h, L.cell);
      k_tag_ulap<<<D.nblocks, kBlock, 0, h->stream>>>(leveld(h, level), D, (const double *)h->Q.p, threshold, T, cover,
                                                      n1);
    } else {
      Decomp D = decomp(h, L.coarse);
      k_tag_rte<<<D.nblocks, kBlock, 0, h->stream>>>(leveld(h, level), D, fields(h), threshold, T, cover, n1);
    }
    k_tag_buffer<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, h->stream>>>(T, cover, out, n0, n1, buffer);
    h->launch_count += 2;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(mask, out, n, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFreeAsync(buf, h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "bsam_tag_level");
  return BSAM_OK;
}

int bsam_vcycle(bsam_hier h) {
  if (!h) return fail(BSAM_ERR_ARG, "null hierarchy");
  int rc = set_device(h);
  if (rc || (rc = ensure_f32(h))) return rc;
  if (mixed(h)) {   // the correction cycle's right-hand side
    launch_consistent(h);
    launch_residual(h, 2);
  } else {
    reset_force(h);
  }
  if ((rc = launch_iteration(h, 2))) return rc;
  CK(cudaStreamSynchronize(h->stream));
  return BSAM_OK;
}

static int finish_solve(bsam_hier h, bool on_device, double *res_hist, int hist_cap, int *vcycles,
                        double *final_rel, int64_t *visible_cells);

int bsam_solve_cycles(bsam_hier h, double *res_hist, int hist_cap, int *vcycles, double *final_rel,
                      int64_t *visible_cells) {
  if (!h) return fail(BSAM_ERR_ARG, "null hierarchy");
  int rc = set_device(h);
  if (rc) return rc;
  if ((rc = ensure_f32(h))) return rc;
  int nactive = 0;
  bool on_device = false;
  if (h->tuned[mixed(h) ? 1 : 0] && !host_loop() && build_solve_graph(h)) {
    // the whole solve in one graph launch (once the smoother is tuned)
    CK(cudaGraphLaunch(h->sexec, h->stream));
    h->solve_graphs++;
    if ((rc = read_state(h, &nactive))) return rc;
    on_device = true;
    return finish_solve(h, on_device, res_hist, hist_cap, vcycles, final_rel, visible_cells);
  }
  if (!mixed(h)) reset_force(h);
  for (int k = 1; k <= h->nlev; ++k) launch_fill(h, k);
  launch_residual(h, 0);
  CK(cudaGetLastError());
  if ((rc = read_state(h, &nactive))) return rc;
  if (nactive && mixed(h)) {
    // the history starts with the reference's own initial residual; the
    // first correction's right-hand side is the consistent hierarchy's
    launch_consistent(h);
    launch_residual(h, 2);
  }
  // every instance iterates until its own stop test fails; a converged
  // instance of a batch is frozen (its stores are predicated off) while the
  // others continue.  The loop runs on the device when the runtime can build
  // its WHILE graph, else one graph launch per V-cycle with a host check.
  if (nactive && (rc = autotune(h))) return rc;
  if (nactive && !host_loop() && build_while_graph(h)) {
    CK(cudaGraphLaunch(h->wexec, h->stream));
    if ((rc = read_state(h, &nactive))) return rc;
    on_device = true;
  }
  if (nactive && (rc = build_graph(h))) return rc;
  while (nactive) {
    CK(cudaGraphLaunch(h->gexec, h->stream));
    h->graph_launches++;
    if ((rc = read_state(h, &nactive))) return rc;
  }
  return finish_solve(h, on_device, res_hist, hist_cap, vcycles, final_rel, visible_cells);
}

// the results of a solve: residual histories and V-cycle counts to the host,
// every instance active again for eager operations
static int finish_solve(bsam_hier h, bool on_device, double *res_hist, int hist_cap, int *vcycles,
                        double *final_rel, int64_t *visible_cells) {
  h->res_hist.resize((size_t)h->ninst * h->hist_stride);
  h->res_iters.resize(h->ninst);
  h->res_acc.assign(h->acc_host, h->acc_host + h->ninst);
  CK(cudaMemcpyAsync(h->res_hist.data(), h->hist.p, sizeof(double) * h->res_hist.size(), cudaMemcpyDeviceToHost,
                     h->stream));
  CK(cudaMemcpyAsync(h->res_iters.data(), h->iters.p, sizeof(int) * h->ninst, cudaMemcpyDeviceToHost, h->stream));
  // eager operations after the solve act on every instance again
  CK(cudaMemcpyAsync(h->active.p, h->ones.p, sizeof(int) * h->ninst, cudaMemcpyDeviceToDevice, h->stream));
  if (h->act_mode == kActChunk) CK(cudaMemsetAsync(h->cact.p, 1, h->cact.n, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (on_device) h->while_bodies += *std::max_element(h->res_iters.begin(), h->res_iters.end());
  return bsam_batch_result(h, 0, res_hist, hist_cap, vcycles, final_rel, visible_cells);
}

int bsam_batch_result(bsam_hier h, int inst, double *res_hist, int hist_cap, int *vcycles, double *final_rel,
                      int64_t *visible_cells) {
  if (!h) return fail(BSAM_ERR_ARG, "null hierarchy");
  if (inst < 0 || inst >= h->ninst) return fail(BSAM_ERR_ARG, "instance out of range");
  if (h->res_iters.empty()) return fail(BSAM_ERR_STATE, "no solve has run on this hierarchy");
  const int it = h->res_iters[inst];
  for (int i = 0; res_hist && i <= it && i < hist_cap; ++i) res_hist[i] = h->res_hist[(size_t)inst * h->hist_stride + i];
  if (vcycles) *vcycles = it;
  if (final_rel) *final_rel = h->res_acc[inst].out[3];
  if (visible_cells) *visible_cells = (int64_t)h->res_acc[inst].out[4];
  return BSAM_OK;
}

int bsam_batch_set_stop(bsam_hier h, int inst, int max_vcycles, double rel_tol) {
  if (!h) return fail(BSAM_ERR_ARG, "null hierarchy");
  if (inst < 0 || inst >= h->ninst) return fail(BSAM_ERR_ARG, "instance out of range");
  if (max_vcycles < 0 || !(rel_tol >= 0)) return fail(BSAM_ERR_ARG, "invalid stop test");
  int rc = set_device(h);
  if (rc) return rc;
  h->hir[inst].max_vcycles = max_vcycles;
  h->hir[inst].rel_tol = rel_tol;
  return upload_stops(h);
}

int bsam_composite_mean(bsam_hier h, double *mean, double *area) {
  double out[4];
  (void)out;
  if (!h) return fail(BSAM_ERR_ARG, "null hierarchy");
  int rc = set_device(h);
  if (rc) return rc;
  Fields f = fields(h);
  int o = 0;
  std::vector<int> starts;
  for (int k = h->root; k <= h->nlev; ++k) {
    const LevelPlan &L = h->lev[k];
    Decomp D = decomp(h, L.cell);
    starts.push_back(o);
    k_sums<<<D.nblocks, kBlock, 0, h->stream>>>(leveld(h, k), D, f, h->partials.p + 4 * o);
    o += D.nblocks;
  }
  CK(cudaGetLastError());
  std::vector<double> part((size_t)4 * o);
  CK(cudaMemcpyAsync(part.data(), h->partials.p, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  double tot = 0, ar = 0;
  int li = 0;
  for (int k = h->root; k <= h->nlev; ++k, ++li) {
    const LevelPlan &L = h->lev[k];
    const double da = L.hx * L.hy;
    double su = 0, nv = 0;
    for (int b = starts[li]; b < starts[li] + L.cell.nblocks; ++b) {
      su = su + part[4 * b];
      nv = nv + part[4 * b + 3];
    }
    tot = tot + su * da;
    ar = ar + nv * da;
  }
  if (mean) *mean = tot / std::max(ar, 2.2250738585072014e-308);
  if (area) *area = ar;
  return BSAM_OK;
}

int bsam_mass_check(bsam_hier h, double out[4]) {
  if (!h || !out) return fail(BSAM_ERR_ARG, "null argument");
  int rc = set_device(h);
  if (rc) return rc;
  Fields f = fields(h);
  int o = 0;
  std::vector<int> starts;
  for (int k = h->root; k <= h->nlev; ++k) {
    const LevelPlan &L = h->lev[k];
    Decomp D = decomp(h, L.cell);
    starts.push_back(o);
    k_sums<<<D.nblocks, kBlock, 0, h->stream>>>(leveld(h, k), D, f, h->partials.p + 4 * o);
    o += D.nblocks;
  }
  CK(cudaGetLastError());
  std::vector<double> part((size_t)4 * o);
  CK(cudaMemcpyAsync(part.data(), h->partials.p, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, h->stream));
  // boundary flux (perimeter-sized): computed on the host from downloaded
  // boundary rows of Q, in the reference's loop order
  std::vector<double> Qh(h->n_q);
  CK(cudaMemcpyAsync(Qh.data(), h->Q.p, sizeof(double) * h->n_q, cudaMemcpyDeviceToHost, h->stream));
  std::vector<double> DeWh(h->DeW.n), DnSh(h->DnS.n);
  std::vector<uint8_t> flh(h->flags.n);
  CK(cudaMemcpyAsync(DeWh.data(), h->DeW.p, sizeof(double) * DeWh.size(), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(DnSh.data(), h->DnS.p, sizeof(double) * DnSh.size(), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(flh.data(), h->flags.p, flh.size(), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  double lhs = 0, scale = 0, rhs = 0;
  int li = 0;
  for (int k = h->root; k <= h->nlev; ++k, ++li) {
    const LevelPlan &L = h->lev[k];
    const double da = L.hx * L.hy, hx = L.hx, hy = L.hy;
    double sm = 0, sa = 0;
    for (int b = starts[li]; b < starts[li] + L.cell.nblocks; ++b) {
      sm = sm + part[4 * b + 1];
      sa = sa + part[4 * b + 2];
    }
    lhs = lhs + sm * da;
    scale = scale + sa * da;
    for (int p = L.p0; p < L.p1; ++p) {
      const int32_t *r = h->hpatches.data() + (size_t)p * PDN;
      const int mx = r[PD_MX], my = r[PD_MY];
      auto Q = [&](int i, int j) { return Qh[r[PD_QOFF] + (i - 1) + (size_t)(j - 1) * (mx + 2)]; };
      auto cov = [&](int i, int j) { return flh[r[PD_COFF] + (i - 1) + (size_t)(j - 1) * mx] & 1; };
      const double *DeW = DeWh.data() + r[PD_DEWOFF], *DnS = DnSh.data() + r[PD_DNSOFF];
      if (r[PD_BCW] > 0) { double fl = 0; for (int j = 1; j <= my; ++j) if (!cov(1, j)) fl = fl + DeW[(size_t)(j - 1) * (mx + 1)] * (Q(1, j + 1) - Q(2, j + 1)) / hx; rhs = rhs + fl * hy; }
      if (r[PD_BCE] > 0) { double fl = 0; for (int j = 1; j <= my; ++j) if (!cov(mx, j)) fl = fl + DeW[mx + (size_t)(j - 1) * (mx + 1)] * (Q(mx + 2, j + 1) - Q(mx + 1, j + 1)) / hx; rhs = rhs + fl * hy; }
      if (r[PD_BCS] > 0) { double fl = 0; for (int i = 1; i <= mx; ++i) if (!cov(i, 1)) fl = fl + DnS[i - 1] * (Q(i + 1, 1) - Q(i + 1, 2)) / hy; rhs = rhs + fl * hx; }
      if (r[PD_BCN] > 0) { double fl = 0; for (int i = 1; i <= mx; ++i) if (!cov(i, my)) fl = fl + DnS[(i - 1) + (size_t)my * mx] * (Q(i + 1, my + 2) - Q(i + 1, my + 1)) / hy; rhs = rhs + fl * hx; }
    }
  }
  out[0] = lhs;
  out[1] = rhs;
  out[2] = lhs - rhs;
  double m = std::max(std::max(scale, std::fabs(lhs)), std::max(std::fabs(rhs), 2.2250738585072014e-308));
  out[3] = std::fabs(lhs - rhs) / m;
  return BSAM_OK;
}

int bsam_save_state(bsam_hier h) {
  if (!h) return fail(BSAM_ERR_ARG, "null hierarchy");
  int rc = set_device(h);
  if (rc) return rc;
  if (!h->saveQ.p && ((rc = h->saveQ.alloc(h->Q.n)) || (rc = h->saveQC.alloc(h->QC.n)) || (rc = h->saveF.alloc(h->F.n))))
    return rc;
  CK(cudaMemcpyAsync(h->saveQ.p, h->Q.p, sizeof(double) * h->Q.n, cudaMemcpyDeviceToDevice, h->stream));
  if (h->QC.n) CK(cudaMemcpyAsync(h->saveQC.p, h->QC.p, sizeof(double) * h->QC.n, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(h->saveF.p, h->F.p, sizeof(double) * h->F.n, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return BSAM_OK;
}

int bsam_restore_state(bsam_hier h) {
  if (!h) return fail(BSAM_ERR_ARG, "null hierarchy");
  if (!h->saveQ.p) return fail(BSAM_ERR_STATE, "no saved state");
  int rc = set_device(h);
  if (rc) return rc;
  CK(cudaMemcpyAsync(h->Q.p, h->saveQ.p, sizeof(double) * h->Q.n, cudaMemcpyDeviceToDevice, h->stream));
  if (h->QC.n) CK(cudaMemcpyAsync(h->QC.p, h->saveQC.p, sizeof(double) * h->QC.n, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(h->F.p, h->saveF.p, sizeof(double) * h->F.n, cudaMemcpyDeviceToDevice, h->stream));
  return BSAM_OK;
}

int bsam_launch_count(bsam_hier h, int64_t *count) {
  if (!h || !count) return fail(BSAM_ERR_ARG, "null argument");
  *count = h->launch_count + h->graph_launches * h->kernels_per_cycle + h->while_bodies * (h->kernels_per_cycle + 1) +
           h->solve_graphs * h->preamble_kernels;
  return BSAM_OK;
}

int bsam_relax_tuning(bsam_hier h, int precision, int32_t *cells_per_thread, int cap) {
  if (!h || !cells_per_thread) return fail(BSAM_ERR_ARG, "null argument");
  if (precision != 0 && precision != 1) return fail(BSAM_ERR_ARG, "precision must be 0 or 1");
  const std::vector<int> &rn = h->relax_n[precision];
  for (int k = 1; k <= h->nlev && k <= cap; ++k)
    cells_per_thread[k - 1] = h->tuned[precision] && (int)rn.size() > k ? rn[k] : -1;
  return BSAM_OK;
}

int bsam_stream(bsam_hier h, void **stream) {
  if (!h || !stream) return fail(BSAM_ERR_ARG, "null argument");
  *stream = (void *)h->stream;
  return BSAM_OK;
}

int bsam_kernels_per_vcycle(bsam_hier h, int64_t *count) {
  if (!h || !count) return fail(BSAM_ERR_ARG, "null argument");
  int rc = set_device(h);
  if (rc || (rc = build_graph(h))) return rc;
  *count = h->kernels_per_cycle;
  return BSAM_OK;
}

int bsam_time_relax(bsam_hier h, int level, int reps, double *us) {
  if (!h || !us || level < 2 || level > h->nlev || reps < 1) return fail(BSAM_ERR_ARG, "bad argument");
  int rc = set_device(h);
  if (rc || (rc = ensure_f32(h))) return rc;
  if (!h->tuned[mixed(h) ? 1 : 0]) return fail(BSAM_ERR_STATE, "bsam_time_relax: the smoother is not tuned yet");
  const int ns = std::max(h->opts.npre, 1);
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  const int64_t before = h->launch_count;
  if (mixed(h)) launch_relax<float>(h, level, ns, false, true);
  else launch_relax<double>(h, level, ns, false, true);
  h->launch_count = before;
  cudaGraph_t g = nullptr;
  CK(cudaStreamEndCapture(h->stream, &g));
  cudaGraphExec_t ge = nullptr;
  cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
  cudaEvent_t a = nullptr, b = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  for (int i = 0; i < 3 && e == cudaSuccess; ++i) e = cudaGraphLaunch(ge, h->stream);
  if (e == cudaSuccess) e = cudaEventRecord(a, h->stream);
  for (int i = 0; i < reps && e == cudaSuccess; ++i) e = cudaGraphLaunch(ge, h->stream);
  if (e == cudaSuccess) e = cudaEventRecord(b, h->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float ms = 0;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (ge) cudaGraphExecDestroy(ge);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "bsam_time_relax");
  *us = 1e3 * (double)ms / ((double)reps * 2 * ns);
  return BSAM_OK;
}

int bsam_profile_vcycles(bsam_hier h, int ncycles, int level, double ms[BSAM_NKINDS], int64_t launches[BSAM_NKINDS],
                         double bytes[BSAM_NKINDS]) {
  if (!h || !ms || !launches || !bytes || ncycles < 1 || level < 0 || level > h->nlev)
    return fail(BSAM_ERR_ARG, "bad argument");
  int rc = set_device(h);
  if (rc) return rc;
  for (int i = 0; i < BSAM_NKINDS; ++i) { ms[i] = 0; launches[i] = 0; bytes[i] = 0; }
  if ((rc = ensure_f32(h))) return rc;
  if (mixed(h)) {
    launch_consistent(h);
    launch_residual(h, 2);
  } else {
    reset_force(h);
  }
  if ((rc = autotune(h))) return rc;
  h->profiling = true;
  h->profile_level = level;
  h->recs.clear();
  for (int c = 0; c < ncycles && !rc; ++c) rc = launch_iteration(h, 2);
  h->profiling = false;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  for (auto &r : h->recs) {
    float t = 0;
    if (e == cudaSuccess && !rc) {
      cudaEventElapsedTime(&t, r.a, r.b);
      ms[r.kind] += t;
      launches[r.kind] += 1;
      bytes[r.kind] += r.bytes;
    }
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  h->recs.clear();
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "profile sync");
  return BSAM_OK;
}

}  // extern "C"
