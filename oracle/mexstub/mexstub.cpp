/*
 * Host harness for the reference's own mex sources -- TEST INFRASTRUCTURE.
 *
 * Implements the handful of MATLAB C API calls that the reference's gateway
 * and TV sources use, plus a C entry point per mexFunction so that Python
 * tests can drive them through ctypes.  mexErrMsgTxt unwinds back to the
 * harness with an error message, as MATLAB aborts the mex call.
 */
#include "mex.h"

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

struct mxArray_tag {
  mxClassID cls;
  std::vector<mwSize> dims;
  std::vector<unsigned char> data;
  std::vector<std::string> names;
  std::vector<mxArray *> fields;
};

static size_t elsize(mxClassID c) {
  return c == mxDOUBLE_CLASS ? 8 : (c == mxSINGLE_CLASS ? 4 : 0);
}
static size_t numel(const mxArray *a) {
  size_t n = 1;
  for (mwSize d : a->dims) n *= d;
  return n;
}

extern "C" {
double *mxGetPr(const mxArray *a) { return (double *)a->data.data(); }
void *mxGetData(const mxArray *a) { return (void *)a->data.data(); }
double mxGetScalar(const mxArray *a) {
  if (a->cls == mxDOUBLE_CLASS) return ((const double *)a->data.data())[0];
  if (a->cls == mxSINGLE_CLASS) return ((const float *)a->data.data())[0];
  return 0;
}
size_t mxGetM(const mxArray *a) { return a->dims.empty() ? 0 : a->dims[0]; }
size_t mxGetN(const mxArray *a) {
  size_t n = 1;
  for (size_t i = 1; i < a->dims.size(); i++) n *= a->dims[i];
  return n;
}
size_t mxGetNumberOfElements(const mxArray *a) { return numel(a); }
const mwSize *mxGetDimensions(const mxArray *a) { return a->dims.data(); }
mxClassID mxGetClassID(const mxArray *a) { return a->cls; }
// stand-in arrays are always real
bool mxIsComplex(const mxArray *) { return false; }
mxArray *mxGetField(const mxArray *s, mwIndex, const char *name) {
  for (size_t i = 0; i < s->names.size(); i++)
    if (s->names[i] == name) return s->fields[i];
  return nullptr;
}
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls,
                              mxComplexity) {
  mxArray *a = new mxArray_tag;
  a->cls = cls;
  a->dims.assign(dims, dims + ndim);
  /* MATLAB keeps at least two dimensions and pads with 1s when asked */
  while (a->dims.size() < 3) a->dims.push_back(1);
  a->data.assign(numel(a) * elsize(cls), 0);
  return a;
}
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls,
                               mxComplexity c) {
  mwSize d[2] = {m, n};
  mxArray *a = mxCreateNumericArray(2, d, cls, c);
  a->dims.resize(2);
  return a;
}
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c) {
  return mxCreateNumericMatrix(m, n, mxDOUBLE_CLASS, c);
}
mxArray *mxCreateStructMatrix(mwSize, mwSize, int nfields, const char **names) {
  mxArray *a = new mxArray_tag;
  a->cls = mxSTRUCT_CLASS;
  a->dims = {1, 1};
  for (int i = 0; i < nfields; i++) {
    a->names.push_back(names[i]);
    a->fields.push_back(nullptr);
  }
  return a;
}
void mxSetField(mxArray *s, mwIndex, const char *name, mxArray *v) {
  for (size_t i = 0; i < s->names.size(); i++)
    if (s->names[i] == name) {
      s->fields[i] = v;
      return;
    }
  s->names.push_back(name);
  s->fields.push_back(v);
}
mxArray *mxCreateDoubleScalar(double v) {
  mxArray *a = mxCreateDoubleMatrix(1, 1, mxREAL);
  *(double *)a->data.data() = v;
  return a;
}
int mexPrintf(const char *fmt, ...) {
  (void)fmt;
  return 0;
}
int mexEvalString(const char *) { return 0; }
void mexErrMsgTxt(const char *msg) { throw std::runtime_error(msg); }

/* ---- harness API used from Python (ctypes) ---- */
mxArray *stub_numeric(int cls, int ndim, const long long *dims) {
  std::vector<mwSize> d(dims, dims + ndim);
  mxArray *a = new mxArray_tag;
  a->cls = (mxClassID)cls;
  a->dims = d;
  a->data.assign(numel(a) * elsize(a->cls), 0);
  return a;
}
mxArray *stub_struct(void) {
  mxArray *a = new mxArray_tag;
  a->cls = mxSTRUCT_CLASS;
  a->dims = {1, 1};
  return a;
}
void stub_struct_set(mxArray *s, const char *name, mxArray *v) {
  s->names.push_back(name);
  s->fields.push_back(v);
}
void *stub_data(mxArray *a) { return a->data.data(); }
int stub_ndim(mxArray *a) { return (int)a->dims.size(); }
long long stub_dim(mxArray *a, int i) { return (long long)a->dims[i]; }
int stub_class(mxArray *a) { return (int)a->cls; }
void stub_free(mxArray *a) {
  if (!a) return;
  for (mxArray *f : a->fields) stub_free(f);
  delete a;
}
}

/* renamed mexFunctions of the reference sources (see build_ref.sh); weak so
 * that the stub also links into libraries without them (the tests of this
 * repository's own gateways) */
__attribute__((weak)) void ref_mex_ax(int, mxArray *[], int, const mxArray *[]);
__attribute__((weak)) void ref_mex_atx(int, mxArray *[], int, const mxArray *[]);
__attribute__((weak)) void ref_mex_tv2d(int, mxArray *[], int, const mxArray *[]);
__attribute__((weak)) void ref_mex_tv3d(int, mxArray *[], int, const mxArray *[]);

typedef void (*mex_fn)(int, mxArray *[], int, const mxArray *[]);

/* Calls any mexFunction; returns 0, or 1 with the mexErrMsgTxt text. */
extern "C" int stub_call_fn(void *fn, int nlhs, mxArray **plhs, int nrhs,
                            const mxArray **prhs, char *err, int errlen) {
  for (int i = 0; i < nlhs; i++) plhs[i] = nullptr;
  try {
    if (!fn) throw std::runtime_error("mexFunction not linked");
    ((mex_fn)fn)(nlhs, plhs, nrhs, prhs);
  } catch (const std::exception &e) {
    if (err && errlen > 0) {
      std::strncpy(err, e.what(), (size_t)errlen - 1);
      err[errlen - 1] = 0;
    }
    return 1;
  }
  return 0;
}

extern "C" mxArray *stub_get_field(mxArray *s, const char *name) {
  return mxGetField(s, 0, name);
}

/* which: 0 Ax_cone_gpu, 1 Atx_cone_gpu, 2 imgTVGradMin, 3 imgTVGradMin3D.
 * Returns 0, or 1 with the mexErrMsgTxt text in err. */
extern "C" int stub_call(int which, int nlhs, mxArray **plhs, int nrhs,
                         const mxArray **prhs, char *err, int errlen) {
  for (int i = 0; i < nlhs; i++) plhs[i] = nullptr;
  try {
    mex_fn f = which == 0   ? ref_mex_ax
               : which == 1 ? ref_mex_atx
               : which == 2 ? ref_mex_tv2d
               : which == 3 ? ref_mex_tv3d
                            : nullptr;
    if (!f) throw std::runtime_error("mexFunction not linked");
    f(nlhs, plhs, nrhs, prhs);
  } catch (const std::exception &e) {
    if (err && errlen > 0) {
      std::strncpy(err, e.what(), (size_t)errlen - 1);
      err[errlen - 1] = 0;
    }
    return 1;
  }
  return 0;
}

/* Adapter with the oracle driver's TV signature (nz==1 -> imgTVGradMin,
 * else imgTVGradMin3D, img_old always passed, as ASD_POCS_cuda.m:156-163). */
extern "C" int ref_tv_for_driver(const double *in, double *out, int nx, int ny,
                                 int nz, double alpha, int n, int pos,
                                 const double *old, int nthreads) {
  (void)nthreads;
  const bool is3d = nz >= 2;
  long long dims[3] = {nx, ny, nz};
  const int nd = is3d ? 3 : 2;
  const size_t N = (size_t)nx * ny * nz;
  mxArray *img = stub_numeric(mxDOUBLE_CLASS, nd, dims);
  mxArray *img0 = stub_numeric(mxDOUBLE_CLASS, nd, dims);
  std::memcpy(stub_data(img), in, N * sizeof(double));
  std::memcpy(stub_data(img0), old, N * sizeof(double));
  long long one[2] = {1, 1};
  mxArray *a = stub_numeric(mxDOUBLE_CLASS, 2, one);
  mxArray *it = stub_numeric(mxDOUBLE_CLASS, 2, one);
  mxArray *ps = stub_numeric(mxDOUBLE_CLASS, 2, one);
  *(double *)stub_data(a) = alpha;
  *(double *)stub_data(it) = n;
  *(double *)stub_data(ps) = pos;
  const mxArray *prhs[5] = {img, a, it, ps, img0};
  mxArray *plhs[1] = {nullptr};
  char err[256];
  int rc = stub_call(is3d ? 3 : 2, 1, plhs, 5, prhs, err, sizeof err);
  if (rc == 0 && plhs[0])
    std::memcpy(out, stub_data(plhs[0]), N * sizeof(double));
  else
    rc = 1;
  stub_free(img);
  stub_free(img0);
  stub_free(a);
  stub_free(it);
  stub_free(ps);
  stub_free(plhs[0]);
  return rc;
}
