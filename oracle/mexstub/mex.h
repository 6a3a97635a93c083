/*
 * Minimal stand-in for MATLAB's mex.h so that the reference's gateway and TV
 * sources (src/AxAtx/*_main_test.cpp, src/tvmin/imgTVGradMin*.cpp) compile
 * for the host as part of the oracle build (oracle/build_ref.sh).
 * Test infrastructure only: it implements just the calls those files make.
 */
#ifndef ASDPOCS_MEXSTUB_H
#define ASDPOCS_MEXSTUB_H
#include <stddef.h>

typedef size_t mwSize;
typedef size_t mwIndex;
typedef ptrdiff_t mwSignedIndex;
typedef enum {
  mxUNKNOWN_CLASS = 0,
  mxDOUBLE_CLASS,
  mxSINGLE_CLASS,
  mxSTRUCT_CLASS
} mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef struct mxArray_tag mxArray;

#ifdef __cplusplus
extern "C" {
#endif

double *mxGetPr(const mxArray *a);
void *mxGetData(const mxArray *a);
double mxGetScalar(const mxArray *a);
size_t mxGetM(const mxArray *a);
size_t mxGetN(const mxArray *a);
size_t mxGetNumberOfElements(const mxArray *a);
const mwSize *mxGetDimensions(const mxArray *a);
mxClassID mxGetClassID(const mxArray *a);
bool mxIsComplex(const mxArray *a);
mxArray *mxGetField(const mxArray *s, mwIndex i, const char *name);
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c);
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls,
                               mxComplexity c);
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls,
                              mxComplexity c);
mxArray *mxCreateStructMatrix(mwSize m, mwSize n, int nfields,
                              const char **names);
void mxSetField(mxArray *s, mwIndex i, const char *name, mxArray *v);
mxArray *mxCreateDoubleScalar(double v);
int mexPrintf(const char *fmt, ...);
int mexEvalString(const char *cmd);
void mexErrMsgTxt(const char *msg);
#ifdef __cplusplus
}
#endif
#endif
