/*
 * mex.h -- a minimal stand-in for the MATLAB MEX API, for testing mex/rtmc_mex.c where
 * neither MATLAB nor Octave is installed.  TEST INFRASTRUCTURE ONLY.
 *
 * mxArray is backed by plain host memory: real double / uint32 / char matrices, 1x1
 * structs with named fields and cells.  mexErrMsgIdAndTxt unwinds to the mex_stub_call
 * that started the gateway (as MATLAB's error does), and records the identifier and the
 * message.  Only the functions rtmc_mex.c uses are provided, with the MATLAB signatures.
 */
#ifndef MEX_STUB_H
#define MEX_STUB_H

#include <stddef.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef size_t mwSize;
typedef size_t mwIndex;
typedef enum { mxUNKNOWN_CLASS = 0, mxCELL_CLASS, mxSTRUCT_CLASS, mxCHAR_CLASS, mxDOUBLE_CLASS, mxUINT32_CLASS } mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef struct mxArray_tag mxArray;

/* the gateway */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);

/* MATLAB API subset */
mxArray *mxGetField(const mxArray *s, mwIndex i, const char *name);
void mxSetField(mxArray *s, mwIndex i, const char *name, mxArray *value);
mxArray *mxGetCell(const mxArray *c, mwIndex i);
bool mxIsEmpty(const mxArray *a);
bool mxIsDouble(const mxArray *a);
bool mxIsComplex(const mxArray *a);
bool mxIsChar(const mxArray *a);
bool mxIsCell(const mxArray *a);
bool mxIsStruct(const mxArray *a);
size_t mxGetNumberOfElements(const mxArray *a);
size_t mxGetM(const mxArray *a);
size_t mxGetN(const mxArray *a);
double *mxGetPr(const mxArray *a);
void *mxGetData(const mxArray *a);
double mxGetScalar(const mxArray *a);
int mxGetString(const mxArray *a, char *buf, mwSize n);
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID c, mxComplexity x);
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity x);
mxArray *mxCreateDoubleScalar(double v);
mxArray *mxCreateStructMatrix(mwSize m, mwSize n, int nfields, const char **names);
void mxDestroyArray(mxArray *a);
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
int mexAtExit(void (*fn)(void));

/* test driver entry points (not MATLAB API) */
mxArray *mex_stub_cell(mwSize n);
void mex_stub_set_cell(mxArray *c, mwIndex i, mxArray *v);
mxArray *mex_stub_string(const char *s);
mxArray *mex_stub_struct(void);
mxArray *mex_stub_doubles(mwSize m, mwSize n, const double *data);
/* runs mexFunction; 0 on return, 1 when it raised (mex_stub_error() gives "id: message") */
int mex_stub_call(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs);
const char *mex_stub_error(void);
int mex_stub_class(const mxArray *a);
void mex_stub_run_atexit(void);
long mex_stub_live(void); /* arrays created and not yet destroyed */

#ifdef __cplusplus
}
#endif

#endif
