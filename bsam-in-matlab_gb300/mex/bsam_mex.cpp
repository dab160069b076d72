// bsam_mex.cpp -- MEX gateway between MATLAB and libbsam_dev.so.
//
// One MEX function, bsam_mex(cmd, ...), dispatches to the C-ABI of
// include/bsam_dev.h.  It is what the reference's ebSolveCycles.m calls when
// its Device option is set (a Device parameter added to ebOptions.m, and a
// branch at the top of ebSolveCycles.m that flattens the hierarchy once per
// structural change, uploads it, solves and writes Q back).  Status codes
// become MATLAB errors with the
// identifiers bsam:device:<code>, in the style of the reference's
// error('pkg:id', msg) calls.
//
// Build where MATLAB is installed:
//   mex -I<repo>/include bsam_mex.cpp -L<dir of libbsam_dev.so> -lbsam_dev
#include "mex.h"
#include "bsam_dev.h"
#include <string>
#include <vector>

static bsam_ctx g_ctx = nullptr;
static void check(int rc) {
  if (rc == BSAM_OK) return;
  static const char *names[] = {"ok", "arg", "cuda", "nomem", "state", "nodev"};
  std::string id = std::string("bsam:device:") + names[rc < 6 ? rc : 2];
  mexErrMsgIdAndTxt(id.c_str(), "%s", bsam_last_error());
}
static void at_exit() { if (g_ctx) bsam_ctx_destroy(g_ctx); g_ctx = nullptr; }
template <class T> static const T *ptr(const mxArray *s, const char *f, int64_t *n) {
  const mxArray *a = mxGetField(s, 0, f);
  *n = (int64_t)mxGetNumberOfElements(a);
  return static_cast<const T *>(mxGetData(a));
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
  std::string cmd = mxArrayToString(prhs[0]);
  if (cmd == "upload") {                       // (T, device, opts) -> handle
    if (!g_ctx) { check(bsam_ctx_create((int)mxGetScalar(prhs[2]), &g_ctx)); mexAtExit(at_exit); }
    const mxArray *T = prhs[1];
    bsam_hier_desc d = {};
    int64_t n;
    d.nlev = (int32_t)mxGetScalar(mxGetField(T, 0, "nlev"));
    d.root_idx = (int32_t)mxGetScalar(mxGetField(T, 0, "rootIdx"));
    d.levels = ptr<int32_t>(T, "levels", &n);
    d.patches = ptr<int32_t>(T, "patches", &n); d.npatch = (int32_t)(n / 36);
    d.hs = ptr<double>(T, "hs", &n);
    d.Q = ptr<double>(T, "Q", &d.n_q);        d.F = ptr<double>(T, "F", &d.n_cells);
    d.FTrue = ptr<double>(T, "FTrue", &n);    d.CC = ptr<double>(T, "CC", &n);
    d.InvDiagS = ptr<double>(T, "InvDiagS", &n);
    d.DeW = ptr<double>(T, "DeW", &d.n_dew);  d.DnS = ptr<double>(T, "DnS", &d.n_dns);
    d.QC = ptr<double>(T, "QC", &d.n_qc);     d.bcg = ptr<double>(T, "bcg", &d.n_bcg);
    d.cfd = ptr<double>(T, "cfd", &d.n_cfd);  d.pcoef = ptr<double>(T, "pcoef", &d.n_pcoef);
    d.covered = ptr<uint8_t>(T, "covered", &n);
    d.same = ptr<int32_t>(T, "same", &n);     d.n_same = n / 2;
    d.ring = ptr<int32_t>(T, "ring", &n);     d.n_ring = n / 2;
    d.win = ptr<int32_t>(T, "win", &d.n_win);
    d.fp = ptr<int32_t>(T, "fp", &n);         d.n_fp = n / 2;
    d.corr = ptr<int32_t>(T, "corr", &d.n_corr);
    d.Ainv = ptr<double>(T, "Ainv", &n);      d.bcRhs = ptr<double>(T, "bcRhs", &n);
    d.ncoarse = (int32_t)n;
    d.singular = (int32_t)mxGetScalar(mxGetField(T, 0, "singular"));
    const mxArray *o = prhs[3];
    bsam_solve_opts so = {(int32_t)mxGetScalar(mxGetField(o, 0, "NPre")),
                          (int32_t)mxGetScalar(mxGetField(o, 0, "NPost")),
                          mxGetScalar(mxGetField(o, 0, "Omega")),
                          (int32_t)mxGetScalar(mxGetField(o, 0, "lif")),
                          (int32_t)mxGetScalar(mxGetField(o, 0, "MassCorrection")),
                          (int32_t)mxGetScalar(mxGetField(o, 0, "MaxVCycles")),
                          mxGetScalar(mxGetField(o, 0, "RelTol")), 0};
    bsam_hier h;
    check(bsam_hier_upload(g_ctx, &d, &so, &h));
    plhs[0] = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
    *(uint64_t *)mxGetData(plhs[0]) = (uint64_t)(uintptr_t)h;
  } else if (cmd == "solveCycles") {           // handle -> [hist, it, rel, vis]
    bsam_hier h = (bsam_hier)(uintptr_t)(*(uint64_t *)mxGetData(prhs[1]));
    double hist[1024]; int it; double rel; int64_t vis;
    check(bsam_solve_cycles(h, hist, 1024, &it, &rel, &vis));
    plhs[0] = mxCreateDoubleMatrix(1, it + 1, mxREAL);
    for (int i = 0; i <= it; ++i) mxGetPr(plhs[0])[i] = hist[i];
    plhs[1] = mxCreateDoubleScalar(it); plhs[2] = mxCreateDoubleScalar(rel);
    plhs[3] = mxCreateDoubleScalar((double)vis);
  } else if (cmd == "getField" || cmd == "setField") {
    bsam_hier h = (bsam_hier)(uintptr_t)(*(uint64_t *)mxGetData(prhs[1]));
    std::string f = mxArrayToString(prhs[2]);
    static const char *names[] = {"Q", "F", "FTrue", "QC", "CC", "InvDiagS", "DeW", "DnS", "pcoef", "cfD", "bcg",
                                  "Ainv", "bcRhs", "Uo", "Uoo"};
    int which = -1;
    for (int i = 0; i < 15; ++i) if (f == names[i]) which = i;   // BSAM_FIELD_* order
    if (cmd == "setField") {
      check(bsam_set_field(h, which, mxGetPr(prhs[3]), (int64_t)mxGetNumberOfElements(prhs[3])));
    } else {
      const int64_t n = (int64_t)mxGetScalar(prhs[3]);
      plhs[0] = mxCreateDoubleMatrix(n, 1, mxREAL);
      check(bsam_get_field(h, which, mxGetPr(plhs[0]), n));
    }
  } else if (cmd == "tag") {                   // handle, level, 'ulap'|'rte', thr, buffer, n0, n1 -> logical mask
    bsam_hier h = (bsam_hier)(uintptr_t)(*(uint64_t *)mxGetData(prhs[1]));
    std::string ind = mxArrayToString(prhs[3]);
    const int n0 = (int)mxGetScalar(prhs[6]), n1 = (int)mxGetScalar(prhs[7]);
    std::vector<uint8_t> m((size_t)n0 * n1);
    check(bsam_tag_level(h, (int)mxGetScalar(prhs[2]), ind == "rte" ? 1 : 0, mxGetScalar(prhs[4]),
                         (int)mxGetScalar(prhs[5]), n0, n1, m.data()));
    plhs[0] = mxCreateLogicalMatrix(n0, n1);   // MATLAB column-major from the i-major mask
    mxLogical *L = mxGetLogicals(plhs[0]);
    for (int i = 0; i < n0; ++i)
      for (int j = 0; j < n1; ++j) L[i + (size_t)j * n0] = m[(size_t)i * n1 + j];
  } else if (cmd == "pRhs") {                  // handle, scheme (0 BE, 1 BDF2), Dt, f (cells or [])
    bsam_hier h = (bsam_hier)(uintptr_t)(*(uint64_t *)mxGetData(prhs[1]));
    const mxArray *f = prhs[4];
    check(bsam_parabolic_rhs(h, (int)mxGetScalar(prhs[2]), mxGetScalar(prhs[3]),
                             mxIsEmpty(f) ? nullptr : mxGetPr(f), (int64_t)mxGetNumberOfElements(f)));
  } else if (cmd == "pPush") {                 // after each step's solve
    check(bsam_history_push((bsam_hier)(uintptr_t)(*(uint64_t *)mxGetData(prhs[1]))));
  } else if (cmd == "free") {
    check(bsam_hier_free((bsam_hier)(uintptr_t)(*(uint64_t *)mxGetData(prhs[1]))));
  } else {
    mexErrMsgIdAndTxt("bsam:device:arg", "unknown command %s", cmd.c_str());
  }
}
