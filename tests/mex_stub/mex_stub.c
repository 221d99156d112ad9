/* Plain-memory implementation of tests/mex_stub/mex.h.  TEST INFRASTRUCTURE ONLY. */
#define _POSIX_C_SOURCE 200809L
#include "mex.h"

#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MAX_FIELDS 64

struct mxArray_tag {
    mxClassID cls;
    size_t m, n;
    void *data;                  /* numeric / char data, or mxArray * [m n] of a cell */
    int nfields;
    char *names[MAX_FIELDS];     /* 1x1 struct */
    mxArray *values[MAX_FIELDS];
};

static jmp_buf g_jump;
static int g_in_call = 0;
static char g_error[1024];
static void (*g_atexit)(void) = NULL;
static long g_live = 0;

static mxArray *make(mxClassID c, size_t m, size_t n, size_t elem)
{
    mxArray *a = (mxArray *)calloc(1, sizeof *a);
    a->cls = c;
    a->m = m;
    a->n = n;
    if (m * n * elem > 0) a->data = calloc(m * n, elem);
    ++g_live;
    return a;
}

mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID c, mxComplexity x)
{
    (void)x;
    return make(c, m, n, c == mxUINT32_CLASS ? 4 : 8);
}
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity x) { return mxCreateNumericMatrix(m, n, mxDOUBLE_CLASS, x); }
mxArray *mxCreateDoubleScalar(double v)
{
    mxArray *a = make(mxDOUBLE_CLASS, 1, 1, 8);
    *(double *)a->data = v;
    return a;
}
mxArray *mex_stub_doubles(mwSize m, mwSize n, const double *data)
{
    mxArray *a = make(mxDOUBLE_CLASS, m, n, 8);
    if (m * n > 0) memcpy(a->data, data, m * n * 8);
    return a;
}
mxArray *mex_stub_string(const char *s)
{
    size_t k = strlen(s);
    mxArray *a = make(mxCHAR_CLASS, 1, k, 1);
    if (k) memcpy(a->data, s, k);
    return a;
}
mxArray *mex_stub_cell(mwSize n) { return make(mxCELL_CLASS, 1, n, sizeof(mxArray *)); }
void mex_stub_set_cell(mxArray *c, mwIndex i, mxArray *v) { ((mxArray **)c->data)[i] = v; }
mxArray *mex_stub_struct(void) { return make(mxSTRUCT_CLASS, 1, 1, 0); }
mxArray *mxCreateStructMatrix(mwSize m, mwSize n, int nfields, const char **names)
{
    mxArray *s = make(mxSTRUCT_CLASS, m, n, 0);
    for (int i = 0; i < nfields && i < MAX_FIELDS; ++i) {
        s->names[i] = strdup(names[i]);
        s->values[i] = NULL;
    }
    s->nfields = nfields;
    return s;
}

void mxSetField(mxArray *s, mwIndex i, const char *name, mxArray *value)
{
    (void)i;
    for (int k = 0; k < s->nfields; ++k)
        if (strcmp(s->names[k], name) == 0) {
            if (s->values[k]) mxDestroyArray(s->values[k]);
            s->values[k] = value;
            return;
        }
    if (s->nfields < MAX_FIELDS) {
        s->names[s->nfields] = strdup(name);
        s->values[s->nfields++] = value;
    }
}

mxArray *mxGetField(const mxArray *s, mwIndex i, const char *name)
{
    if (!s || s->cls != mxSTRUCT_CLASS || i != 0) return NULL;
    for (int k = 0; k < s->nfields; ++k)
        if (strcmp(s->names[k], name) == 0) return s->values[k];
    return NULL;
}

mxArray *mxGetCell(const mxArray *c, mwIndex i)
{
    if (!c || c->cls != mxCELL_CLASS || i >= c->m * c->n) return NULL;
    return ((mxArray **)c->data)[i];
}

void mxDestroyArray(mxArray *a)
{
    if (!a) return;
    if (a->cls == mxCELL_CLASS)
        for (size_t i = 0; i < a->m * a->n; ++i) mxDestroyArray(((mxArray **)a->data)[i]);
    for (int k = 0; k < a->nfields; ++k) {
        free(a->names[k]);
        mxDestroyArray(a->values[k]);
    }
    free(a->data);
    free(a);
    --g_live;
}

bool mxIsEmpty(const mxArray *a) { return !a || a->m * a->n == 0; }
bool mxIsDouble(const mxArray *a) { return a && a->cls == mxDOUBLE_CLASS; }
bool mxIsComplex(const mxArray *a) { (void)a; return false; }
bool mxIsChar(const mxArray *a) { return a && a->cls == mxCHAR_CLASS; }
bool mxIsCell(const mxArray *a) { return a && a->cls == mxCELL_CLASS; }
bool mxIsStruct(const mxArray *a) { return a && a->cls == mxSTRUCT_CLASS; }
size_t mxGetNumberOfElements(const mxArray *a) { return a ? a->m * a->n : 0; }
size_t mxGetM(const mxArray *a) { return a ? a->m : 0; }
size_t mxGetN(const mxArray *a) { return a ? a->n : 0; }
double *mxGetPr(const mxArray *a) { return a && a->cls == mxDOUBLE_CLASS ? (double *)a->data : NULL; }
void *mxGetData(const mxArray *a) { return a ? a->data : NULL; }
double mxGetScalar(const mxArray *a) { return mxIsDouble(a) && a->m * a->n > 0 ? ((double *)a->data)[0] : 0.0; }
int mex_stub_class(const mxArray *a) { return a ? (int)a->cls : -1; }
long mex_stub_live(void) { return g_live; }

int mxGetString(const mxArray *a, char *buf, mwSize n)
{
    if (!mxIsChar(a) || n == 0) return 1;
    size_t k = a->m * a->n;
    if (k + 1 > n) return 1;
    memcpy(buf, a->data, k);
    buf[k] = 0;
    return 0;
}

void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...)
{
    va_list ap;
    int k = snprintf(g_error, sizeof g_error, "%s: ", id);
    va_start(ap, fmt);
    vsnprintf(g_error + k, sizeof g_error - (size_t)k, fmt, ap);
    va_end(ap);
    if (g_in_call) longjmp(g_jump, 1);
    fprintf(stderr, "%s\n", g_error);
    abort();
}

int mexAtExit(void (*fn)(void))
{
    g_atexit = fn;
    return 0;
}

void mex_stub_run_atexit(void)
{
    if (g_atexit) g_atexit();
    g_atexit = NULL;
}

int mex_stub_call(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs)
{
    g_error[0] = 0;
    g_in_call = 1;
    if (setjmp(g_jump)) {
        g_in_call = 0;
        return 1;
    }
    mexFunction(nlhs, plhs, nrhs, prhs);
    g_in_call = 0;
    return 0;
}

const char *mex_stub_error(void) { return g_error; }
