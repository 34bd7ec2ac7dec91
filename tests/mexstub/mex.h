/* Minimal stand-in for MATLAB's mex.h (declarations only): lets the tests compile the
   MEX gateway sources of the integration guide for a syntax and ABI check. */
#include <stddef.h>
#include <stdint.h>
typedef struct mxArray_tag mxArray;
typedef size_t mwSize;
typedef size_t mwIndex;
typedef enum { mxREAL = 0 } mxComplexity;
mwSize mxGetN(const mxArray*);
mwSize mxGetM(const mxArray*);
mwIndex* mxGetJc(const mxArray*);
mwIndex* mxGetIr(const mxArray*);
double* mxGetDoubles(const mxArray*);
void* mxMalloc(mwSize);
mwSize mxGetNumberOfElements(const mxArray*);
void mexErrMsgIdAndTxt(const char*, const char*, ...);
int mxIsSparse(const mxArray*);
int mxIsDouble(const mxArray*);
int mxGetString(const mxArray*, char*, mwSize);
int mxIsEmpty(const mxArray*);
double mxGetScalar(const mxArray*);
int mxIsInf(double);
mxArray* mxCreateDoubleMatrix(mwSize, mwSize, mxComplexity);
int mexAtExit(void (*)(void));
typedef enum { mxDOUBLE_CLASS = 6, mxSINGLE_CLASS = 7 } mxClassID;
typedef float mxSingle;
mxArray* mxCreateNumericMatrix(mwSize, mwSize, mxClassID, mxComplexity);
mxSingle* mxGetSingles(const mxArray*);
void mxFree(void*);
