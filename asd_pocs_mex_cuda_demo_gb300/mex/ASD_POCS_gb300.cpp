// MATLAB gateway: [m_res, out] = ASD_POCS_gb300(P, para) -- the whole
// ASD_POCS_cuda.m reconstruction on the GPU in one call.
//
// Same arguments and outputs as utilities/ASD_POCS_cuda.m (P: (na*nb) x nv
// double; para: nx ny nz SO OD vxlsize detsize na nb phi_vec and the
// optional maxnumIter numOfgradients alpha alpha_red beta beta_red r_max
// epsilon stopRelChg m0 I0), but the sinogram goes to the GPU once and every
// iteration runs there (FP32 images, FP64 step-control scalars), instead of
// one host round trip per view and per TV call.  out has IterationNum,
// dataTolerance, alpha, beta and, with para.I0, RMSE.  Build (MATLAB):
//   mex -output ASD_POCS_gb300 ASD_POCS_gb300.cpp -I<include> -L<lib> -lasdpocs_gb300
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "asdpocs_gb300.h"
#include "mex.h"

static double field(const mxArray *para, const char *name, double dflt,
                    bool required) {
  const mxArray *f = mxGetField(para, 0, name);
  if (!f || mxGetNumberOfElements(f) == 0) {
    if (required) {
      char msg[96];
      snprintf(msg, sizeof msg, "Error input argument parameter.%s!", name);
      mexErrMsgTxt(msg);
    }
    return dflt;
  }
  return mxGetScalar(f);
}

// A real double array (MATLAB's default class), as the reconstruction reads
// its elements as doubles.
static bool real_double(const mxArray *a) {
  return mxGetClassID(a) == mxDOUBLE_CLASS && !mxIsComplex(a);
}

// Optional image field (para.m0, para.I0): NULL when absent or empty, else it
// must be a real double array of nx*ny*nz elements.
static const double *image_field(const mxArray *para, const char *name, size_t N) {
  const mxArray *f = mxGetField(para, 0, name);
  if (!f || mxGetNumberOfElements(f) == 0) return NULL;
  if (!real_double(f) || mxGetNumberOfElements(f) != N) {
    char msg[112];
    snprintf(msg, sizeof msg, "parameter.%s must be a real double array of nx*ny*nz elements!",
             name);
    mexErrMsgTxt(msg);
  }
  return mxGetPr(f);
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
  if (nrhs != 2) mexErrMsgTxt("Error usage! [m_res,out] = ASD_POCS_gb300(P, para)");
  const mxArray *P = prhs[0], *para = prhs[1];
  if (!real_double(P)) mexErrMsgTxt("P must be a real double matrix");
  asdpocs_geometry g;
  g.nx = (int)field(para, "nx", 0, true);
  g.ny = (int)field(para, "ny", 0, true);
  g.nz = (int)field(para, "nz", 0, true);
  g.na = (int)field(para, "na", 0, true);
  g.nb = (int)field(para, "nb", 0, true);
  g.SO = field(para, "SO", 0, true);
  g.OD = field(para, "OD", 0, true);
  g.vxlsize = field(para, "vxlsize", 0, true);
  g.detsize = field(para, "detsize", 0, true);
  const mxArray *phi = mxGetField(para, 0, "phi_vec");
  if (!phi) mexErrMsgTxt("Error input argument parameter.phi_vec!");
  if (!real_double(phi)) mexErrMsgTxt("parameter.phi_vec must be a real double vector!");
  g.nv = (int)mxGetN(P);
  if ((int)mxGetNumberOfElements(phi) != g.nv)
    mexErrMsgTxt("Size of Projection and phi_vec mismatch!");  // ASD_POCS_cuda.m:97-100
  // one column of na*nb rays per view: the reference's P(:,ii) - proj
  // (ASD_POCS_cuda.m:121) fails on any other row count
  if (g.na <= 0 || g.nb <= 0 || mxGetM(P) != (size_t)g.na * (size_t)g.nb)
    mexErrMsgTxt("Matrix dimensions must agree: P must have na*nb rows!");
  asdpocs_options o;
  asdpocs_options_default(&o);
  o.maxnumIter = (int)field(para, "maxnumIter", o.maxnumIter, false);
  o.numOfgradients = (int)field(para, "numOfgradients", o.numOfgradients, false);
  o.alpha = field(para, "alpha", o.alpha, false);
  o.alpha_red = field(para, "alpha_red", o.alpha_red, false);
  o.beta = field(para, "beta", o.beta, false);
  o.beta_red = field(para, "beta_red", o.beta_red, false);
  o.r_max = field(para, "r_max", o.r_max, false);
  o.epsilon = field(para, "epsilon", o.epsilon, false);
  o.stopRelChg = field(para, "stopRelChg", o.stopRelChg, false);
  const size_t N = (size_t)g.nx * g.ny * g.nz;
  const double *m0 = image_field(para, "m0", N);
  const double *I0 = image_field(para, "I0", N);
  mwSize dims[3] = {(mwSize)g.nx, (mwSize)g.ny, (mwSize)g.nz};
  plhs[0] = mxCreateNumericArray(3, dims, mxDOUBLE_CLASS, mxREAL);
  std::vector<double> rmse((size_t)(o.maxnumIter > 0 ? o.maxnumIter : 1));
  asdpocs_stats st;
  const int rc = ASD_POCS_cuda(
      mxGetPr(P), mxGetPr(phi), &g, &o, m0, I0, mxGetPr(plhs[0]), rmse.data(), &st);
  if (rc != 0) mexErrMsgTxt(asdpocs_last_error());
  if (nlhs > 1) {
    const char *names[] = {"IterationNum", "dataTolerance", "beta", "alpha", "RMSE"};
    const int nf = I0 ? 5 : 4;
    plhs[1] = mxCreateStructMatrix(1, 1, nf, names);
    mxSetField(plhs[1], 0, "IterationNum", mxCreateDoubleScalar(st.IterationNum));
    mxSetField(plhs[1], 0, "dataTolerance", mxCreateDoubleScalar(st.dataTolerance));
    mxSetField(plhs[1], 0, "beta", mxCreateDoubleScalar(st.beta));
    mxSetField(plhs[1], 0, "alpha", mxCreateDoubleScalar(st.alpha));
    if (nf == 5) {
      mxArray *r = mxCreateDoubleMatrix((mwSize)st.IterationNum, 1, mxREAL);
      memcpy(mxGetPr(r), rmse.data(), sizeof(double) * (size_t)st.IterationNum);
      mxSetField(plhs[1], 0, "RMSE", r);
    }
  }
}
