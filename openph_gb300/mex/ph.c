/*
 * ph.c — MATLAB MEX gateway for libopenph_gb300: the same call as the
 * reference's `ph` MEX (src/matlab/ph/ph.cu:11-92),
 *
 *   [low, ess, err_linf, err_lone, err_redu, err_ess, time_track, num_iters]
 *       = ph(algstr, int32 r, int32 c, int32 m, int32 col_width, int32 low_true)
 *
 * forwarding to openph() of include/openph.h.  Built only where MATLAB is
 * installed:
 *
 *   mex -I<repo>/include ph.c -L<repo>/openph_gb300 -lopenph_gb300
 *
 * Unlike the reference gateway this checks its argument counts and types and
 * raises a MATLAB error on failure instead of printing.
 */
#include <string.h>

#include "mex.h"
#include "openph.h"

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    if (nrhs != 6) mexErrMsgIdAndTxt("openph:ph", "ph needs 6 inputs: algstr, r, c, m, col_width, low_true");
    if (nlhs > 8) mexErrMsgIdAndTxt("openph:ph", "ph has at most 8 outputs");
    if (!mxIsChar(prhs[0])) mexErrMsgIdAndTxt("openph:ph", "algstr must be a string");
    for (int k = 1; k < 6; k++)
        if (!mxIsInt32(prhs[k])) mexErrMsgIdAndTxt("openph:ph", "r, c, m, col_width and low_true must be int32");
    char algstr[64];
    if (mxGetString(prhs[0], algstr, sizeof(algstr)) != 0) mexErrMsgIdAndTxt("openph:ph", "algstr too long");
    int *rows = (int *)mxGetData(prhs[1]);
    int *cols = (int *)mxGetData(prhs[2]);
    int m = (int)mxGetScalar(prhs[3]);
    int col_width = (int)mxGetScalar(prhs[4]);
    int *low_true = (int *)mxGetData(prhs[5]);
    int nnz = (int)mxGetNumberOfElements(prhs[1]);
    if ((int)mxGetNumberOfElements(prhs[2]) != nnz) mexErrMsgIdAndTxt("openph:ph", "r and c differ in length");
    if ((int)mxGetNumberOfElements(prhs[5]) != m) mexErrMsgIdAndTxt("openph:ph", "low_true must have m entries");

    plhs[0] = mxCreateNumericMatrix(1, m, mxINT32_CLASS, mxREAL);
    plhs[1] = mxCreateNumericMatrix(1, m, mxINT32_CLASS, mxREAL);
    for (int k = 2; k < 7; k++) plhs[k] = mxCreateNumericMatrix(1, m + 1, mxSINGLE_CLASS, mxREAL);
    plhs[7] = mxCreateNumericMatrix(1, 1, mxINT32_CLASS, mxREAL);
    float *f[5];
    for (int k = 0; k < 5; k++) {
        f[k] = (float *)mxGetData(plhs[k + 2]);
        for (int i = 0; i < m + 1; i++) f[k][i] = k == 4 ? 0.0f : -1.0f;
    }
    int rc = oph_openph(algstr, rows, cols, m, col_width, low_true, nnz, (int *)mxGetData(plhs[0]),
                        (int *)mxGetData(plhs[1]), f[0], f[1], f[2], f[3], f[4], (int *)mxGetData(plhs[7]), 0);
    if (rc != OPH_OK) mexErrMsgIdAndTxt("openph:ph", "openph: %s", oph_status_string(rc));
}
