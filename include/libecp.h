/*
 * libecp.h -- handle interface of the drop-in library (replaces chrr/libECP
 * src/libecp.h:6-29; same symbols, argument order and semantics).
 *
 * libECP_init keeps the caller's geometry and basis arrays by pointer (they
 * must outlive the handle) and copies the ECP terms (src/libecp.c:68-127).
 * calculateECPIntegrals computes every (shell pair, ECP centre) block on the
 * GPU, then hands the blocks to the callback in the reference's order
 * (centre C, atom A, atom B >= A, shell s1 of A, shell s2 of B -- s2 >= s1 when
 * A == B -- type-1 block then type-2 block), each IJK(la) x IJK(lb) row-major
 * in libint Cartesian order and freed after the callback returns
 * (src/libecp.c:256-397).  Return value: 0 ok; 1 (type 1) or 2 (type 2) when
 * a large-grid quadrature exhausted its levels -- the reference's codes for an
 * integration error (src/libecp.h:23-27).  The reference then uses a freed
 * table and aborts in practice; here that quadrature keeps its full-grid
 * estimate and every block is still handed out.  -1: engine error (no GPU,
 * allocation).  LIBECP_GB300_MODE=fast in the environment runs the blocks on
 * the batched FP64 engine (see getIntegrals.h).
 */
#ifndef LIBECP_H
#define LIBECP_H 1

#ifdef __cplusplus
extern "C" {
#endif

typedef struct _libECPHandle libECPHandle;

/* The reference's typedef names the parameters (A, B, C, sa, sb, la, lb,
 * shifta, shiftb, I, p) but calls it as below (src/libecp.c:372,
 * src/getIntegrals.c:23-25); the ABI is the same nine ints, a double* and a
 * void*, and the meaning follows the call site. */
typedef void (*ECPCallback)(int A, int sa, int la, int shifta,
                            int B, int sb, int lb, int shiftb,
                            int C, double *I, void *p);

/* The reference's header names parameters 4 and 5 (KECP, lECP) but its
 * definition reads them as (lECP, KECP) (src/libecp.c:55), and getIntegrals
 * passes them in that order; this declaration follows the definition.
 * n: nuclear-derivative order 0, 1 or 2, as the reference: blocks of the
 * shells with l shifted by (shifta, shiftb) and coefficients times zeta^shift
 * (src/libecp.c:240-374).
 * lmax / shellOrdering: the caller's Cartesian ordering of shells 0..lmax
 * (NULL = libint default), refused as the reference refuses it when lmax is
 * too small (src/libecp.c:152-166).
 * Returns NULL on failure. */
libECPHandle *libECP_init(int nrAtoms, double *geometry,
                          int *shellsECP, int *lECP, int *KECP,
                          double *nECP, double *dECP, double *aECP,
                          int *shellsBS, int *lBS, int *KBS,
                          double *dBS, double *aBS,
                          int n, int lmax, int *shellOrdering,
                          int largeGridOrder, double tolerance, double accuracy);

int calculateECPIntegrals(libECPHandle *h, ECPCallback cb, void *args);

void libECP_free(libECPHandle *h);

#ifdef __cplusplus
}
#endif
#endif /* LIBECP_H */
