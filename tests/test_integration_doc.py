"""The MEX gateway source (bsam-in-matlab_gb300/mex/bsam_mex.cpp) compiles
against include/bsam_dev.h (a syntax check with g++: MATLAB's mex.h is not
installed, so the handful of MEX API functions the gateway calls are
declared here with plain C types)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MEX_DECLS = r'''
#include <stddef.h>
#include <stdint.h>
typedef struct mxArray_tag mxArray;
typedef bool mxLogical;
typedef enum { mxUINT64_CLASS = 13 } mxClassID;
typedef enum { mxREAL = 0 } mxComplexity;
extern "C" {
char *mxArrayToString(const mxArray *);
mxArray *mxGetField(const mxArray *, size_t, const char *);
size_t mxGetNumberOfElements(const mxArray *);
void *mxGetData(const mxArray *);
double mxGetScalar(const mxArray *);
double *mxGetPr(const mxArray *);
mxArray *mxCreateNumericMatrix(size_t, size_t, mxClassID, mxComplexity);
mxArray *mxCreateDoubleMatrix(size_t, size_t, mxComplexity);
mxArray *mxCreateDoubleScalar(double);
mxArray *mxCreateLogicalMatrix(size_t, size_t);
mxLogical *mxGetLogicals(const mxArray *);
bool mxIsEmpty(const mxArray *);
void mexErrMsgIdAndTxt(const char *, const char *, ...);
int mexAtExit(void (*)(void));
}
'''


def test_mex_gateway_compiles_against_the_header(tmp_path):
    if shutil.which('g++') is None:
        pytest.skip('g++ not available')
    src = os.path.join(ROOT, 'bsam-in-matlab_gb300', 'mex', 'bsam_mex.cpp')
    code = open(src).read()
    assert 'bsam_hier_upload' in code and 'bsam_solve_cycles' in code
    (tmp_path / 'mex.h').write_text(MEX_DECLS)
    out = subprocess.run(['g++', '-std=c++17', '-fsyntax-only', '-Wall', '-Werror', '-I', str(tmp_path), '-I',
                          os.path.join(ROOT, 'include'), src],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr[-3000:]
