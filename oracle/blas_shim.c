/* Forwards the plain Fortran BLAS/LAPACK names the ITensor reference calls
 * (dgemm_, dsyev_, ...) to the scipy-bundled OpenBLAS, whose symbols carry a
 * scipy_ prefix. Every Fortran argument is a pointer, so a forwarder passes a
 * fixed number of pointer slots through; the callee reads only its own.
 * Test infrastructure: linked only into oracle/_ref/ref_golden. */
#include <complex.h>
#define P void*
#define A20 P a1,P a2,P a3,P a4,P a5,P a6,P a7,P a8,P a9,P a10,P a11,P a12,P a13,P a14,P a15,P a16,P a17,P a18,P a19,P a20
#define V20 a1,a2,a3,a4,a5,a6,a7,a8,a9,a10,a11,a12,a13,a14,a15,a16,a17,a18,a19,a20
#define FWD_VOID(n) extern void scipy_##n##_(A20); void n##_(A20) { scipy_##n##_(V20); }
#define FWD_DBL(n)  extern double scipy_##n##_(A20); double n##_(A20) { return scipy_##n##_(V20); }
FWD_VOID(daxpy) FWD_VOID(dscal) FWD_VOID(dgemm) FWD_VOID(dgemv) FWD_VOID(zgemm) FWD_VOID(zgemv)
FWD_VOID(dsyev) FWD_VOID(dgesdd) FWD_VOID(dgesvd) FWD_VOID(zgesvd) FWD_VOID(zgesdd)
FWD_VOID(dgeqrf) FWD_VOID(dorgqr) FWD_VOID(zgeqrf) FWD_VOID(zungqr) FWD_VOID(dgesv) FWD_VOID(zgesv)
FWD_VOID(zheev) FWD_VOID(dsygv) FWD_VOID(dgeev) FWD_VOID(zgeev)
FWD_DBL(ddot) FWD_DBL(dnrm2) FWD_DBL(dlange) FWD_DBL(zlange)
extern double _Complex scipy_zdotc_(A20);
double _Complex zdotc_(A20) { return scipy_zdotc_(V20); }
