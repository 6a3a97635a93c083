// MATLAB gateway: I2 = imgTVGradMin3D(I, alpha, nTVIter, pos[, I0]) on the GPU.
//
// Drop-in for src/tvmin/imgTVGradMin3D.cpp (FP64 stencil on the GPU through
// the asdpocs_gb300 library).  Build (MATLAB):
//   mex -output imgTVGradMin3D imgTVGradMin3D_gb300.cpp -I<include> -L<lib> -lasdpocs_gb300
#include "asdpocs_gb300.h"
#include "mex.h"

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
  (void)nlhs;
  if (nrhs != 4 && nrhs != 5) {  // imgTVGradMin3D.cpp:21-25
    mexPrintf("usage: I2 = imgTVGradMin3D(I, alpha, nTVIter, pos[, I0])\n");
    return;
  }
  if (mxGetClassID(prhs[0]) != mxDOUBLE_CLASS) {
    mexPrintf("Invalid data format. Please make sure the input image data is in double format.\n");
    return;
  }
  const mwSize *dim = mxGetDimensions(prhs[0]);
  const int Nx = (int)dim[0], Ny = (int)dim[1], Nz = (int)dim[2];
  const double *img_old = NULL;
  if (nrhs == 5) {
    const mwSize *d0 = mxGetDimensions(prhs[4]);
    if ((int)d0[0] != Nx || (int)d0[1] != Ny || (int)d0[2] != Nz) {
      mexPrintf("img0 dimensions do not match with img\n");
      return;
    }
    img_old = mxGetPr(prhs[4]);
  }
  plhs[0] = mxCreateNumericArray(3, dim, mxDOUBLE_CLASS, mxREAL);
  const int rc = imgTVGradMin3D(mxGetPr(prhs[0]), mxGetPr(plhs[0]), Nx, Ny, Nz,
                                mxGetScalar(prhs[1]), (int)mxGetScalar(prhs[2]),
                                (int)mxGetScalar(prhs[3]), img_old);
  if (rc != 0) mexErrMsgTxt(asdpocs_last_error());
}
