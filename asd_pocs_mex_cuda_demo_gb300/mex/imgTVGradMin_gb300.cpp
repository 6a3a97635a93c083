// MATLAB gateway: I2 = imgTVGradMin(I, alpha, nTVIter, pos[, I0]) on the GPU.
//
// Drop-in for src/tvmin/imgTVGradMin.cpp (same arguments, same checks, same
// result up to FP64 rounding of the norm sum), computed by the asdpocs_gb300
// library (FP64 stencil on the GPU).  Build (MATLAB, library in <lib>):
//   mex -output imgTVGradMin imgTVGradMin_gb300.cpp -I<include> -L<lib> -lasdpocs_gb300
#include <string.h>

#include "asdpocs_gb300.h"
#include "mex.h"

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
  (void)nlhs;
  if (nrhs != 4 && nrhs != 5) {  // imgTVGradMin.cpp:19-23
    mexPrintf("usage: I2 = imgTVGradMin(I, alpha, nTVIter, pos[, I0])\n");
    return;
  }
  if (mxGetClassID(prhs[0]) != mxDOUBLE_CLASS) {  // imgTVGradMin.cpp:135-139
    mexPrintf("Invalid data format. Please make sure the input image data is in double format.\n");
    return;
  }
  const int rowN = (int)mxGetM(prhs[0]), colN = (int)mxGetN(prhs[0]);
  const double *img_old = NULL;
  if (nrhs == 5) {
    if ((int)mxGetM(prhs[4]) != rowN || (int)mxGetN(prhs[4]) != colN) {
      mexPrintf("img0 dimensions do not match with img\n");
      return;
    }
    img_old = mxGetPr(prhs[4]);
  }
  plhs[0] = mxCreateDoubleMatrix(rowN, colN, mxREAL);
  const int rc = imgTVGradMin(mxGetPr(prhs[0]), mxGetPr(plhs[0]), rowN, colN,
                              mxGetScalar(prhs[1]), (int)mxGetScalar(prhs[2]),
                              (int)mxGetScalar(prhs[3]), img_old);
  if (rc != 0) mexErrMsgTxt(asdpocs_last_error());
}
