/* empty stand-in for MATLAB matrix.h (declarations live in mex.h) */
