/*
 * bsam_dev.h -- C-ABI of libbsam_dev.so, the GB300 (sm_103a) solve path of
 * the BSAM adaptive FAS V-cycle.
 *
 * The reference (BSAM-in-MATLAB) has one hot path, the pure function
 *     H = ebSolveCycles(H)          EllipticBSAM/src/ebSolveCycles.m:1-80
 *                                   EllipticBSAMTree/src/ebtSolveCycles.m
 * called from ebSolve.m:38,41,52, ebtSolve.m:40,43,54 and, once per time
 * step, ParabolicBSAM/src/ebpSolve.m:50.  A host (the MATLAB MEX gateway,
 * or the Python mirror in bsam-in-matlab_gb300/bsam) flattens H into the
 * tables below once per hierarchy change, uploads them, and replaces each
 * ebSolveCycles call with bsam_solve_cycles.  The arithmetic is IEEE FP64 in
 * the reference's operation order: results match the reference up to the
 * coarsest direct solve, whose sparse LU is replaced by a dense inverse.
 *
 * Conventions: every call returns BSAM_OK (0) or an error code; the message
 * of the most recent failure on the calling thread is bsam_last_error().
 * Arrays are host pointers; field arrays are concatenations of per-patch
 * column-major arrays (x fastest), exactly the reference's layout.  Levels
 * are 1-based like the reference's H.lev{k}.  No call allocates on behalf of
 * the caller beyond what bsam_hier_upload documents.
 */
#ifndef BSAM_DEV_H
#define BSAM_DEV_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes; the MEX gateway maps them to error ids bsam:device:<name> */
#define BSAM_OK 0
#define BSAM_ERR_ARG 1      /* invalid argument or malformed table          */
#define BSAM_ERR_CUDA 2     /* CUDA runtime failure                         */
#define BSAM_ERR_NOMEM 3    /* device memory exhausted                      */
#define BSAM_ERR_STATE 4    /* call not valid in the current state          */
#define BSAM_ERR_NODEV 5    /* no usable sm_103 device                      */

/* fields for bsam_set_field / bsam_get_field */
#define BSAM_FIELD_Q 0      /* padded solution, all levels                  */
#define BSAM_FIELD_F 1      /* working force (cells)                        */
#define BSAM_FIELD_FTRUE 2  /* true source (cells)                          */
#define BSAM_FIELD_QC 3     /* padded coarse shadows (levels >= 2)          */
#define BSAM_FIELD_CC 4     /* reaction coefficient (cells)                 */
#define BSAM_FIELD_INVDIAG 5 /* relaxation diagonal InvDiagS (cells)        */
/* coefficient arrays (incremental upload: the execution plan depends on the
 * hierarchy's structure only, so new coefficients of an unchanged hierarchy
 * -- ebpSetTime.m:11-55 -- replace these arrays without a new upload)     */
#define BSAM_FIELD_DEW 6     /* x-face D                                     */
#define BSAM_FIELD_DNS 7     /* y-face D                                     */
#define BSAM_FIELD_PCOEF 8   /* parent coefficients over each footprint      */
#define BSAM_FIELD_CFD 9     /* coarse interface D                           */
#define BSAM_FIELD_BCG 10    /* boundary data                                */
#define BSAM_FIELD_AINV 11   /* coarsest inverse blocks                      */
#define BSAM_FIELD_BCRHS 12  /* coarsest boundary right-hand side            */
/* BDF2 history of the parabolic driver (cells), resident on the device     */
#define BSAM_FIELD_UO 13     /* u at t_n                                     */
#define BSAM_FIELD_UOO 14    /* u at t_{n-1}                                 */

typedef struct bsam_ctx_s *bsam_ctx;
typedef struct bsam_hier_s *bsam_hier;

/* Flat hierarchy: the reference's H (ebMakeLevel.m, ebBuildOps.m,
 * ebtBuildOps.m, ebGatherParentCoeffs.m, ebCoarsest.m) with patch-local
 * indices made global.  Column layouts of `levels` and `patches` are the
 * LD_* and PD_* enumerations of bsam-in-matlab_gb300/bsam/flat.py.        */
typedef struct {
  int32_t nlev, root_idx, npatch;
  const int32_t *levels;    /* [nlev][8]  n0 n1 p0 p1 cell0 cell1 q0 q1     */
  const double *hs;         /* [nlev][2]  hx hy                             */
  const int32_t *patches;   /* [npatch][36]                                 */
  const double *Q, *F, *FTrue, *QC, *CC, *InvDiagS, *DeW, *DnS;
  const double *bcg;        /* boundary data per patch: W(my) E(my) S(mx) N(mx) */
  const double *cfd;        /* interface D per patch: W(cmy) E(cmy) S(cmx) N(cmx) */
  const double *pcoef;      /* parent coefficients: PDeW, PDnS, PCC per patch */
  const uint8_t *covered;   /* 1 = covered by a finer level (cells)         */
  const int32_t *same;      /* [n_same][2] (src Q, dst Q)                   */
  const int32_t *ring;      /* [n_ring][2] (src Q, dst QC)                  */
  const int32_t *win;       /* [n_win] src Q per parent-window cell         */
  const int32_t *fp;        /* [n_fp][2] (parent Q, parent cell)            */
  const int32_t *corr;      /* [n_corr] target cell per coarse face or -1   */
  const double *Ainv;       /* [ncoarse][ncoarse] row-major coarsest inverse */
  const double *bcRhs;      /* [ncoarse]                                    */
  int64_t n_q, n_cells, n_dew, n_dns, n_qc, n_bcg, n_cfd, n_pcoef;
  int64_t n_same, n_ring, n_win, n_fp, n_corr;
  int32_t ncoarse, singular;  /* coarsest unknowns (all instances), singular flag */
  /* A batch of independent instances (ninst >= 2) solved together: every
   * level k holds the level-k patches of every instance (instance by
   * instance, in instance order -- checked at upload -- all instances
   * sharing the level's cell size); patch_inst
   * [npatch] gives each patch's 0-based instance, inst_root [ninst] each
   * instance's root level, and level 1 holds one patch per instance whose
   * inverse blocks are concatenated in Ainv / bcRhs in instance order.
   * ninst = 0 or 1 is a single hierarchy (patch_inst, inst_root unused). */
  int32_t ninst;
  const int32_t *patch_inst;
  const int32_t *inst_root;
} bsam_hier_desc;

/* Solver options: ebOptions.m:44-73 names (NPre, NPost, Omega, GhostInterp,
 * MassCorrection, MaxVCycles, RelTol) plus the precision form.           */
typedef struct {
  int32_t npre, npost;
  double omega;
  int32_t ghost_interp;     /* 0 = 'qif', 1 = 'lif'                         */
  int32_t mass_correction;  /* MassCorrection                               */
  int32_t max_vcycles;
  double rel_tol;
  int32_t precision;        /* 0 = fp64 (drop-in), 1 = mixed                */
} bsam_solve_opts;

/* Context: one device, one stream.  Replaces nothing in the reference (the
 * MATLAB session); created once by the gateway.  A hierarchy uploaded on a
 * context keeps it alive: bsam_ctx_destroy and bsam_hier_free may come in
 * either order, and the last of them releases the context's stream.      */
int bsam_ctx_create(int device, bsam_ctx *out);
int bsam_ctx_destroy(bsam_ctx ctx);

/* Free and total memory of a device (admission control of the serving
 * loop; no reference counterpart). */
int bsam_device_memory(int device, int64_t *free_bytes, int64_t *total_bytes);

/* Measured issue rate of separate FP64 multiplies and adds on the context's
 * device (the form every kernel of the library uses: no contraction), in
 * 1e9 operations per second: independent chains on every SM, best of three
 * CUDA-event timings.  The denominator of the FP64-bound kernels' roofline
 * (no reference counterpart).                                            */
int bsam_fp64_rate(bsam_ctx ctx, double *gops);

/* Message of the last failed call on this thread ("" if none). */
const char *bsam_last_error(void);

/* Upload a hierarchy (allocates its device arrays and execution plan).
 * Replaces the per-call struct copy of ebSolveCycles(H): called after
 * ebSetup.m:10-69, ebAddLevel.m:6-32 (ebtAddLevel.m), ebpRegrid.m:16-58,
 * ebpSetTime.m:11-55.  Validates every table index before any copy.     */
int bsam_hier_upload(bsam_ctx ctx, const bsam_hier_desc *desc, const bsam_solve_opts *opts,
                     bsam_hier *out);
int bsam_hier_free(bsam_hier h);
int bsam_set_opts(bsam_hier h, const bsam_solve_opts *opts);

/* Whole-field copies host <-> device (n = element count, checked). */
int bsam_set_field(bsam_hier h, int which, const double *host, int64_t n);
int bsam_get_field(bsam_hier h, int which, double *host, int64_t n);

/* ebFillGhosts(H,k) (EllipticBSAM/src/ebFillGhosts.m:17-94). */
int bsam_fill_ghosts(bsam_hier h, int level);

/* Initial guess of a new level by bilinear prolongation of the parent
 * window (ebAddLevel.m:26-31): Q_k interior = prolongBilin(W). */
int bsam_prolong_level(bsam_hier h, int level);

/* The device steps of the hierarchy set-up, deferred: for every level k =
 * 1..nlev in order, the new-level prolongation (ebAddLevel.m:26-31) of the
 * instances whose level k lies above their root, then the ghost fill of
 * level k (ebSetup.m:66, ebAddLevel.m:29-31).  A host that builds the
 * hierarchy without a device (the serving loop's builder processes) uploads
 * the pre-step fields and calls this once; the result equals running the
 * steps as the set-up goes.  No reference counterpart as one call. */
int bsam_setup_levels(bsam_hier h);

/* H = ebSolveCycles(H) (ebSolveCycles.m:8-70): ghost fill, residual r_0,
 * then V-cycles until rel <= RelTol or MaxVCycles.  res_hist receives
 * vcycles+1 max-norm residuals (up to hist_cap).  The solution stays on the
 * device; read it with bsam_get_field(BSAM_FIELD_Q). */
int bsam_solve_cycles(bsam_hier h, double *res_hist, int hist_cap, int *vcycles, double *final_rel,
                      int64_t *visible_cells);

/* Per-instance results of the last bsam_solve_cycles on a batch (instance
 * 0 is what bsam_solve_cycles itself reports).  Every instance runs
 * ebSolveCycles' own loop: it stops at its own RelTol / MaxVCycles and its
 * state then stays frozen while the other instances continue, so each
 * instance's solution and history equal those of a solve of it alone.
 * No reference counterpart (the reference solves one hierarchy per call). */
int bsam_batch_result(bsam_hier h, int inst, double *res_hist, int hist_cap, int *vcycles, double *final_rel,
                      int64_t *visible_cells);

/* Stop test (MaxVCycles, RelTol) of one instance of a batch; bsam_set_opts
 * sets every instance's to the options' values. */
int bsam_batch_set_stop(bsam_hier h, int inst, int max_vcycles, double rel_tol);

/* Parabolic step on the device (ParabolicBSAM, kept resident across steps).
 * bsam_parabolic_rhs: ebpRhs.m:25-47 for scheme 0 = BE, FTrue = f + Uo/Dt,
 * or 1 = BDF2, FTrue = f + (2 Uo - 0.5 Uoo)/Dt, on every cell of the levels
 * at or above the root; f (cells, host) may be NULL for f = 0.
 * bsam_history_push: after a step's solve, Uoo = Uo, Uo = the interior of
 * Q on every level (ebpSolve.m:52-56). */
int bsam_parabolic_rhs(bsam_hier h, int scheme, double dt, const double *f, int64_t n);
int bsam_history_push(bsam_hier h);

/* The BDF2 history across a regrid, device to device (replaces the history
 * part of ebpRegrid.m:16-59 and its transferLevel / conslinInterior /
 * parentFootprint / interiors, :62-162): hn is the new hierarchy (uploaded,
 * solution already transferred), hold the old one, both resident on the same
 * device.  src_old[n = hn's cell count] gives for each cell of hn at or
 * above its root the old hierarchy's cell holding the same cell of the same
 * level, or -1 where the old hierarchy had no patch there (every root cell
 * has one).  With has_uoo, level by level from the root up: Uoo(hn) = the old
 * Uoo where src_old >= 0, else the conservative-linear prolongation of hn's
 * parent-level Uoo over the patch footprint (one-sided slopes at its edges);
 * then Uo(hn) = the interior of hn's Q on every level (ebpRegrid.m:49).  No
 * history value passes through host memory.  Synchronous. */
int bsam_history_transfer(bsam_hier hn, bsam_hier hold, const int32_t *src_old, int64_t n, int has_uoo);

/* Tagging of the finest level on the device (ebTagCluster.m:50-59 'ulap',
 * indicator 0; ebRte.m:14-41 'rte', indicator 1), on the current solution:
 * tag where the indicator exceeds threshold, dilate by `buffer` cells
 * (ebTagCluster.m:113-127) and keep the cells the 8-eroded patch cover
 * allows (ebTagCluster.m:130-141).  mask receives the level's n0 x n1 index
 * space, i-major (mask[i * n1 + j], 0-based), 1 = tagged; the host clusters
 * it.  Single hierarchies only. */
int bsam_tag_level(bsam_hier h, int level, int indicator, double threshold, int buffer, int n0, int n1,
                   uint8_t *mask);

/* One ebVcycle(H, nlev) + ebTransfer(H,0,'filldown') (ebVcycle.m:16-35,
 * ebTransfer.m:73-79), force reset included (ebSolveCycles.m:30-34). */
int bsam_vcycle(bsam_hier h);

/* ebTransfer(H,0,'filldown') alone (ebTransfer.m:73-79): restrict every
 * level into its parent and refill the parent's ghosts, finest first. */
int bsam_filldown(bsam_hier h);

/* ebCompResidual (ebCompResidual.m:15-85): out = {linf, l2, fnorm, rel, ncell}. */
int bsam_comp_residual(bsam_hier h, double out[5]);

/* ebCompositeMean (ebCompositeMean.m:4-23) of the solution. */
int bsam_composite_mean(bsam_hier h, double *mean, double *area);

/* ebMassCheck (ebMassCheck.m:15-66): out = {lhs, flux, defect, rel}. */
int bsam_mass_check(bsam_hier h, double out[4]);

/* Measurement support (no reference counterpart): the CUDA stream the
 * hierarchy's kernels run on (a cudaStream_t), and per-kernel device times
 * of `ncycles` eagerly launched V-cycles, each kernel bracketed by CUDA
 * events on that stream, restricted to the kernels of one level (level 0:
 * all; the residual counts as level 0 only).  kinds: 0 relax, 1 ghost fill,
 * 2 restrict, 3 ring, 4 coarse load, 5 flux corrections, 6 prolong-correct,
 * 7 coarsest, 8 residual; ms[k] = total ms, launches[k], bytes[k] =
 * algorithmic bytes. */
int bsam_stream(bsam_hier h, void **stream);
#define BSAM_NKINDS 9
/* Live cost of one colour pass of level `level`'s smoother in the solve's
 * precision: the npre-sweep relaxation's colour passes (no closing fill)
 * captured as one graph of programmatic-launch-chained kernels, as the
 * solve's graph runs them, replayed `reps` times with CUDA events on the
 * hierarchy's stream; *us = microseconds per pass.  Works on the live state
 * (the caller restores it); the smoother must be tuned (a solve ran).  No
 * counterpart in the reference: measurement. */
int bsam_time_relax(bsam_hier h, int level, int reps, double *us);
int bsam_profile_vcycles(bsam_hier h, int ncycles, int level, double ms[BSAM_NKINDS],
                         int64_t launches[BSAM_NKINDS], double bytes[BSAM_NKINDS]);

/* Device-side snapshot of the solution state (Q, QC, F) and its restore,
 * so repeated solves of one resident hierarchy start from the same state
 * without host traffic (no reference counterpart).  restore is stream-
 * ordered (asynchronous); the first save allocates the snapshot buffers. */
int bsam_save_state(bsam_hier h);
int bsam_restore_state(bsam_hier h);

/* BSAM_SOLVE_LOOP=host in the environment makes bsam_solve_cycles replay a
 * per-V-cycle graph with a host check of the stop tests instead of its
 * device-side loop (a conditional graph node); same kernels and results.
 * For profilers that cannot see kernels inside conditional graphs.       */

/* Kernels launched on this hierarchy so far (eager and graph-replayed). */
int bsam_launch_count(bsam_hier h, int64_t *count);

/* The smoother's launch form per level as the autotuner chose it at the
 * first solve, levels 1..nlev in cells_per_thread[0..nlev-1], for
 * precision 0 (FP64 cycle) or 1 (FP32 correction cycle): 1, 2 or 4 colour
 * cells updated per thread, one launch per colour pass; 3 for one launch
 * per pass of resident blocks that walk the level's chunks, the next
 * chunks' operands in flight during each update; 0 for the whole relaxation
 * (every pass and the closing ghost fill) in one launch of a single
 * thread-block cluster; 5 for the same with the level's solution held in
 * the cluster's distributed shared memory (levels whose Q range fits it);
 * -1 where that cycle has not run yet.  The choice never changes a result
 * bit; BSAM_RELAX_N=0|1|2|3|4|5 in the environment forces one form (5 where
 * it fits, else 1).  No reference counterpart (ebRelaxLevel.m has one loop
 * order).                                                                 */
int bsam_relax_tuning(bsam_hier h, int precision, int32_t *cells_per_thread, int cap);

/* Number of kernels one V-cycle (+ fill-down + residual) launches. */
int bsam_kernels_per_vcycle(bsam_hier h, int64_t *count);

/* Diffuse-domain coefficient sampling on the device (the O(n x segments)
 * part of DiffuseDomainBSAM/src/ddStarfishGeometry.m:140-177): for each of
 * the n points (x[i], y[i]), best[i] <- min(best[i], min_j dd_j) where dd_j
 * is the squared distance to segment j of the closed polygon verts
 * [nverts][2] (x, y interleaved, last vertex = first), computed with the
 * reference's per-segment formula.  best[i] comes in holding the host's
 * starting candidate; the host applies the sign and the square root.  All
 * arrays are host memory; the call is synchronous. */
int bsam_polygon_dist2(bsam_ctx ctx, const double *verts, int nverts, const double *x, const double *y, double *best,
                       int64_t n);

/* Residual norms of one patch on caller-owned device memory, with no device
 * allocation at all.  No counterpart in the reference: it serves callers
 * that cannot call cudaMalloc -- a host that lends the library memory from
 * its own pool (a MATLAB gpuArray, a framework's caching allocator) or code
 * that must not allocate while it runs.  Computes the PLAIN residual
 * r = FTrue - op2d(Q) (ebKernels.m:13-25) over the cells whose `covered`
 * byte is 0 (covered may be NULL) and writes out[0..4] = {linf, l2, fnorm,
 * rel, ncell} (formed as in ebCompResidual.m:66-83) to DEVICE memory `out`.
 * It adds no coarse-fine flux corrections (ebCompResidual.m:40-65), so it
 * equals the reference's composite residual only for a patch that no finer
 * level touches.  The max-norms ignore NaN values, as MATLAB's max does.
 * Q is the padded (mx+2)x(my+2) solution, FTrue/CC/covered mx*my, DeW
 * (mx+1)*my, DnS mx*(my+1), all column-major device arrays; `stream` is a
 * cudaStream_t (NULL = legacy default stream); the call is asynchronous.
 * Its reduction scratch is one static device array of
 * BSAM_NOALLOC_MAX_BLOCKS + 4 doubles (128 KiB) held by every GPU that loads
 * the library until exit, so mx*my is limited to BSAM_NOALLOC_MAX_BLOCKS*256
 * = 4,194,304 cells (BSAM_ERR_ARG beyond).  All calls share that array:
 * calls that overlap on the GPU race and must be serialised by the caller.
 * Each call looks up the array's device address for the current device
 * (valid after a device reset too); the first call on a device may load the
 * library's device code, so make it before any stream capture. */
#define BSAM_NOALLOC_MAX_BLOCKS 16384
int bsam_patch_residual_noalloc(const double *Q, const double *FTrue, const double *DeW, const double *DnS,
                                const double *CC, const uint8_t *covered, int mx, int my, double hx, double hy,
                                double *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* BSAM_DEV_H */
