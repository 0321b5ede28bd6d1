/*
 * Declarations of the MATLAB C Matrix / MEX API functions that
 * nufft_3d_gb300/matlab/nufft3d_mex.c uses, with the documented R2018a
 * (interleaved complex) signatures.  For a compile-only check of the gateway
 * on machines without MATLAB: nothing here is linked or run.
 */
#ifndef NUFFT3D_TEST_MEX_STUB_H
#define NUFFT3D_TEST_MEX_STUB_H
#include <stddef.h>
#include <stdint.h>
#include <stdbool.h>

typedef struct mxArray_tag mxArray;
typedef size_t mwSize;
typedef size_t mwIndex;
typedef enum { mxUNKNOWN_CLASS = 0, mxDOUBLE_CLASS = 6, mxSINGLE_CLASS = 7, mxINT32_CLASS = 12,
               mxUINT64_CLASS = 15 } mxClassID;
typedef enum { mxREAL, mxCOMPLEX } mxComplexity;
typedef struct { float real, imag; } mxComplexSingle;

void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
bool mxIsUint64(const mxArray *a);
bool mxIsSingle(const mxArray *a);
bool mxIsDouble(const mxArray *a);
bool mxIsComplex(const mxArray *a);
bool mxIsEmpty(const mxArray *a);
bool mxIsStruct(const mxArray *a);
size_t mxGetNumberOfElements(const mxArray *a);
size_t mxGetM(const mxArray *a);
double mxGetScalar(const mxArray *a);
int mxGetString(const mxArray *a, char *buf, mwSize len);
uint64_t *mxGetUint64s(const mxArray *a);
int32_t *mxGetInt32s(const mxArray *a);
double *mxGetDoubles(const mxArray *a);
float *mxGetSingles(const mxArray *a);
mxComplexSingle *mxGetComplexSingles(const mxArray *a);
mxArray *mxGetField(const mxArray *s, mwIndex i, const char *name);
void mxSetField(mxArray *s, mwIndex i, const char *name, mxArray *v);
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID c, mxComplexity x);
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID c, mxComplexity x);
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity x);
mxArray *mxCreateDoubleScalar(double v);
mxArray *mxCreateStructMatrix(mwSize m, mwSize n, int nfields, const char **names);
void mxDestroyArray(mxArray *a);
#endif
