/* Test-only helpers of the mock MEX runtime (mex_mock.c). */
#ifndef NUFFT3D_TEST_MEX_MOCK_H
#define NUFFT3D_TEST_MEX_MOCK_H
#include "mex.h"

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);
/* Runs one MEX call; returns 1 if it raised an error (message: mock_last_error). */
int mock_call(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs);
const char *mock_last_error(void);
mxArray *mock_string(const char *s);
#endif
