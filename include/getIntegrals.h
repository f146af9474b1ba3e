/*
 * getIntegrals.h -- one-call interface of the drop-in library (replaces
 * chrr/libECP src/getIntegrals.h:7-13; same symbol and semantics).
 *
 * Accumulates (+=) the ECP matrix elements <a|U|b> of all basis functions into
 * the row-major matrix I (row stride rowdim), upper triangle only (row <= col),
 * Cartesian functions in libint order, AO offsets running over atoms and
 * their shells (src/getIntegrals.c:23-95).  The caller zeroes I.
 *   geometry[3*nrAtoms] (bohr); shellsECP[nrAtoms] ECP shells per atom;
 *   KECP / lECP per ECP shell (terms, channel l); nECP/dECP/aECP per term;
 *   shellsBS[nrAtoms]; lBS / KBS per basis shell; dBS / aBS per primitive
 *   (coefficients used as given).  Defaults: 1024, 1e-12, 1e-14.
 * Returns 0, or 1 if set-up failed (prints "error initializing libECP").  As
 * in the reference, quadrature failures are not reported here; use
 * ecpgb_getIntegrals (libecp_gb300.h) for a status.
 * Engine: the plain FP64 kernels; the environment variable
 * LIBECP_GB300_MODE=fast selects the batched FP64 engine (the same results
 * within 1e-10, several times faster), =mixed the mixed-precision mode.
 */
#ifndef GET_INTEGRALS_H
#define GET_INTEGRALS_H 1

#ifdef __cplusplus
extern "C" {
#endif

int getIntegrals(int nrAtoms, double *geometry,
                 int *shellsECP, int *KECP,
                 int *lECP, double *nECP, double *dECP, double *aECP,
                 int *shellsBS, int *lBS, int *KBS,
                 double *dBS, double *aBS,
                 int largeGridOrder, double tolerance, double accuracy,
                 int rowdim, double *I);

#ifdef __cplusplus
}
#endif
#endif /* GET_INTEGRALS_H */
