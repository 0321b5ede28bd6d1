/*
 * A minimal stand-in for the MATLAB C Matrix / MEX runtime (test
 * infrastructure): just the functions that nufft_3d_gb300/matlab/nufft3d_mex.c
 * calls, with their documented R2018a (interleaved complex) behaviour, so the
 * gateway can be linked and run against libnufft3d.so without MATLAB.
 * mexErrMsgIdAndTxt records the message and unwinds to the caller through
 * mock_call() (longjmp), as MATLAB unwinds a MEX call on error.
 */
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"
#include "mex_mock.h"

struct mxArray_tag {
    mxClassID cls;
    mxComplexity cx;
    size_t ndim;
    size_t dims[4];
    void *data;
    /* struct arrays (1x1 only) */
    int is_struct, nfields;
    char **names;
    mxArray **fields;
    /* char arrays */
    char *str;
};

static jmp_buf *g_jmp = NULL;
static char g_err[512];

const char *mock_last_error(void) { return g_err; }

void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    int n = snprintf(g_err, sizeof g_err, "%s: ", id);
    vsnprintf(g_err + n, sizeof g_err - (size_t)n, fmt, ap);
    va_end(ap);
    if (g_jmp) longjmp(*g_jmp, 1);
    fprintf(stderr, "mex error outside a call: %s\n", g_err);
    exit(3);
}

int mock_call(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs)
{
    jmp_buf jb;
    g_err[0] = 0;
    g_jmp = &jb;
    if (setjmp(jb)) {
        g_jmp = NULL;
        return 1;
    }
    mexFunction(nlhs, plhs, nrhs, prhs);
    g_jmp = NULL;
    return 0;
}

static size_t elem_size(mxClassID c)
{
    switch (c) {
    case mxDOUBLE_CLASS: return 8;
    case mxSINGLE_CLASS: return 4;
    case mxINT32_CLASS: return 4;
    case mxUINT64_CLASS: return 8;
    default: return 1;
    }
}

size_t mxGetNumberOfElements(const mxArray *a)
{
    if (a->str) return strlen(a->str);
    if (a->is_struct) return 1;
    size_t n = 1;
    for (size_t i = 0; i < a->ndim; ++i) n *= a->dims[i];
    return n;
}

mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID c, mxComplexity x)
{
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    a->cls = c;
    a->cx = x;
    a->ndim = ndim < 2 ? 2 : ndim;
    a->dims[0] = a->dims[1] = 1;
    for (size_t i = 0; i < ndim && i < 4; ++i) a->dims[i] = dims[i];
    a->data = calloc(mxGetNumberOfElements(a) ? mxGetNumberOfElements(a) : 1, elem_size(c) * (x == mxCOMPLEX ? 2 : 1));
    return a;
}

mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID c, mxComplexity x)
{
    mwSize d[2] = {m, n};
    return mxCreateNumericArray(2, d, c, x);
}

mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity x) { return mxCreateNumericMatrix(m, n, mxDOUBLE_CLASS, x); }

mxArray *mxCreateDoubleScalar(double v)
{
    mxArray *a = mxCreateDoubleMatrix(1, 1, mxREAL);
    ((double *)a->data)[0] = v;
    return a;
}

mxArray *mxCreateStructMatrix(mwSize m, mwSize n, int nfields, const char **names)
{
    (void)m;
    (void)n;
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    a->is_struct = 1;
    a->ndim = 2;
    a->dims[0] = a->dims[1] = 1;
    a->nfields = nfields;
    a->names = (char **)calloc((size_t)nfields, sizeof(char *));
    a->fields = (mxArray **)calloc((size_t)nfields, sizeof(mxArray *));
    for (int i = 0; i < nfields; ++i) {
        a->names[i] = (char *)malloc(strlen(names[i]) + 1);
        strcpy(a->names[i], names[i]);
    }
    return a;
}

mxArray *mock_string(const char *s)
{
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    a->ndim = 2;
    a->dims[0] = 1;
    a->dims[1] = strlen(s);
    a->str = (char *)malloc(strlen(s) + 1);
    strcpy(a->str, s);
    return a;
}

void mxDestroyArray(mxArray *a)
{
    if (!a) return;
    if (a->is_struct) {
        for (int i = 0; i < a->nfields; ++i) {
            free(a->names[i]);
            mxDestroyArray(a->fields[i]);
        }
        free(a->names);
        free(a->fields);
    }
    free(a->str);
    free(a->data);
    free(a);
}

mxArray *mxGetField(const mxArray *s, mwIndex i, const char *name)
{
    (void)i;
    if (!s || !s->is_struct) return NULL;
    for (int k = 0; k < s->nfields; ++k)
        if (strcmp(s->names[k], name) == 0) return s->fields[k];
    return NULL;
}

void mxSetField(mxArray *s, mwIndex i, const char *name, mxArray *v)
{
    (void)i;
    for (int k = 0; k < s->nfields; ++k)
        if (strcmp(s->names[k], name) == 0) {
            mxDestroyArray(s->fields[k]);
            s->fields[k] = v;
            return;
        }
}

bool mxIsUint64(const mxArray *a) { return !a->str && !a->is_struct && a->cls == mxUINT64_CLASS; }
bool mxIsSingle(const mxArray *a) { return !a->str && !a->is_struct && a->cls == mxSINGLE_CLASS; }
bool mxIsDouble(const mxArray *a) { return !a->str && !a->is_struct && a->cls == mxDOUBLE_CLASS; }
bool mxIsComplex(const mxArray *a) { return a->cx == mxCOMPLEX; }
bool mxIsEmpty(const mxArray *a) { return mxGetNumberOfElements(a) == 0; }
bool mxIsStruct(const mxArray *a) { return a->is_struct != 0; }
size_t mxGetM(const mxArray *a) { return a->dims[0]; }

double mxGetScalar(const mxArray *a)
{
    if (!a->data || mxGetNumberOfElements(a) == 0) return 0;
    switch (a->cls) {
    case mxDOUBLE_CLASS: return ((double *)a->data)[0];
    case mxSINGLE_CLASS: return ((float *)a->data)[0];
    case mxINT32_CLASS: return ((int *)a->data)[0];
    case mxUINT64_CLASS: return (double)((uint64_t *)a->data)[0];
    default: return 0;
    }
}

int mxGetString(const mxArray *a, char *buf, mwSize len)
{
    if (!a->str || len == 0) return 1;
    strncpy(buf, a->str, len - 1);
    buf[len - 1] = 0;
    return strlen(a->str) + 1 > len ? 1 : 0;
}

uint64_t *mxGetUint64s(const mxArray *a) { return a->cls == mxUINT64_CLASS ? (uint64_t *)a->data : NULL; }
int32_t *mxGetInt32s(const mxArray *a) { return a->cls == mxINT32_CLASS ? (int32_t *)a->data : NULL; }
double *mxGetDoubles(const mxArray *a) { return a->cls == mxDOUBLE_CLASS && a->cx == mxREAL ? (double *)a->data : NULL; }
float *mxGetSingles(const mxArray *a) { return a->cls == mxSINGLE_CLASS && a->cx == mxREAL ? (float *)a->data : NULL; }
mxComplexSingle *mxGetComplexSingles(const mxArray *a)
{
    return a->cls == mxSINGLE_CLASS && a->cx == mxCOMPLEX ? (mxComplexSingle *)a->data : NULL;
}

size_t mock_dim(const mxArray *a, int i) { return i < (int)a->ndim ? a->dims[i] : 1; }
size_t mock_ndim(const mxArray *a) { return a->ndim; }
