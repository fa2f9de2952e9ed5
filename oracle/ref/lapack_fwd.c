/* LAPACK/BLAS entry points the reference's matrix_impl.cpp declares,
   forwarded to the copy of OpenBLAS that scipy bundles (it exports them with
   a "scipy_" prefix).  Fortran LP64 calling convention; the trailing hidden
   character-length arguments are passed as 1. */
typedef long flen;
extern int scipy_dgemm_(char*, char*, int*, int*, int*, double*, double*, int*, double*, int*, double*, double*, int*, flen, flen);
extern void scipy_dgetrf_(int*, int*, double*, int*, int*, int*);
extern void scipy_dgetri_(int*, double*, int*, int*, double*, int*, int*);
extern void scipy_dpptrf_(char*, int*, double*, int*, flen);
extern void scipy_dpptri_(char*, int*, double*, int*, flen);
extern void scipy_dsptrd_(char*, int*, double*, double*, double*, double*, int*, flen);
extern void scipy_dopgtr_(char*, int*, double*, double*, double*, int*, double*, int*, flen);
extern void scipy_dsteqr_(char*, int*, double*, double*, double*, int*, double*, int*, flen);
extern void scipy_dpteqr_(char*, int*, double*, double*, double*, int*, double*, int*, flen);

int dgemm_(char* ta, char* tb, int* m, int* n, int* k, double* al, double* a, int* lda, double* b, int* ldb, double* be, double* c, int* ldc)
{ return scipy_dgemm_(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc, 1, 1); }
void dgetrf_(int* m, int* n, double* a, int* lda, int* piv, int* info) { scipy_dgetrf_(m, n, a, lda, piv, info); }
void dgetri_(int* n, double* a, int* lda, int* piv, double* w, int* lw, int* info) { scipy_dgetri_(n, a, lda, piv, w, lw, info); }
void dpptrf_(char* u, int* n, double* a, int* info) { scipy_dpptrf_(u, n, a, info, 1); }
void dpptri_(char* u, int* n, double* a, int* info) { scipy_dpptri_(u, n, a, info, 1); }
void dsptrd_(char* u, int* n, double* a, double* d, double* e, double* tau, int* info) { scipy_dsptrd_(u, n, a, d, e, tau, info, 1); }
void dopgtr_(char* u, int* n, double* a, double* tau, double* q, int* ldq, double* w, int* info) { scipy_dopgtr_(u, n, a, tau, q, ldq, w, info, 1); }
void dsteqr_(char* c, int* n, double* d, double* e, double* z, int* ldz, double* w, int* info) { scipy_dsteqr_(c, n, d, e, z, ldz, w, info, 1); }
void dpteqr_(char* c, int* n, double* d, double* e, double* z, int* ldz, double* w, int* info) { scipy_dpteqr_(c, n, d, e, z, ldz, w, info, 1); }
