// Test harness: exports the gateways of asd_pocs_mex_cuda_demo_gb300/mex
// (compiled with renamed mexFunctions) to ctypes.
#include "mex.h"

void gw_tv2d(int, mxArray *[], int, const mxArray *[]);
void gw_tv3d(int, mxArray *[], int, const mxArray *[]);
void gw_asdpocs(int, mxArray *[], int, const mxArray *[]);

extern "C" void *gw_lookup(int which) {
  switch (which) {
    case 0: return (void *)gw_tv2d;
    case 1: return (void *)gw_tv3d;
    case 2: return (void *)gw_asdpocs;
    default: return nullptr;
  }
}
