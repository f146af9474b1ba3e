/*
 * ecp_oracle.h -- TEST INFRASTRUCTURE ONLY (parity checker and CPU baseline).
 *
 * A plain-C, FP64 restatement of chrr/libECP's integral path: everything from
 * getIntegrals (src/getIntegrals.c:45-95) down to the per-block arithmetic of
 * type1.c / type2.c.  Nothing in the product links this; the tests, the
 * package's smoke check and bench.py's CPU-baseline leg load it via ctypes.
 *
 * Argument meaning everywhere follows getIntegrals (src/getIntegrals.h:7-13):
 * KECP = number of Gaussian terms per ECP shell, lECP = angular momentum of
 * each ECP shell; basis coefficients are used raw.
 */
#ifndef ECP_ORACLE_H
#define ECP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Work counters filled by the oracle while it follows the reference's control
 * flow.  They are implementation-independent (they count what the reference's
 * own loops visit), which is why the algorithmic-flop figure is built on them. */
typedef struct {
  long long blocks;           /* (pair, centre) units that produced a block pair */
  long long ps93_calls;       /* small-grid quadratures                            */
  long long ps93_points;      /* integrand evaluations inside them                 */
  long long ps93_failed;      /* of which did not converge on 383 points           */
  long long psm92_calls;      /* large-grid (fallback) quadratures                 */
  long long psm92_points;
  long long psm92_failed;     /* fallbacks out of levels: the full-grid estimate is
                                 kept (the reference has undefined behaviour)     */
  long long t1_prim_pairs;    /* type-1 primitive pairs                            */
  long long t1_fallback_pp;   /* type-1 primitive pairs that needed the 1023 grid  */
  long long t2_items;         /* (pair, centre, l) type-2 items                    */
  long long t2_fallback_items;/* of which needed the per-primitive fallback        */
  long long t2_fallback_pp;   /* primitive pairs tabulated on the 1023 grid        */
  long long bessel_calls;     /* weighted Bessel evaluations (one argument)        */
  long long bessel_rows;      /* sum over calls of (lmax + 1)                      */
  long long exp_calls;        /* exp() evaluations in tables and integrands        */
  long long table_points;     /* grid points tabulated (F, type-1, fallback)       */
  long long contraction_fma;  /* angular / polynomial contraction multiply-adds    */
  long long stale_reads;      /* fallback quadratures that read a point beyond the
                                 screened end (reference reuses stale buffers)     */
  long long ps93_decisions;   /* small-grid error tests taken (levels with points) */
  long long ps93_divfree_flips;/* of which 16 d < tol 3 n (the GPU's division-free
                                 form) decides otherwise than 16 d / (3 n) < tol  */
} OracleStats;

/* Same semantics as getIntegrals: accumulates (+=) the upper triangle of the
 * Cartesian ECP matrix into I (row stride rowdim).  Only ECP centres with
 * index in [centerLo, centerHi) contribute (use 0, nrAtoms for all).
 * Returns 0 on success, 1 if table set-up failed, 3 for unsupported sizes.
 * A large-grid quadrature that runs out of levels keeps its full-grid
 * estimate and is counted in stats->psm92_failed (the reference has undefined
 * behaviour there and aborts in practice). */
int oracle_getIntegrals(int nrAtoms, const double *geometry,
                        const int *shellsECP, const int *KECP, const int *lECP,
                        const double *nECP, const double *dECP, const double *aECP,
                        const int *shellsBS, const int *lBS, const int *KBS,
                        const double *dBS, const double *aBS,
                        int largeGridOrder, double tolerance, double accuracy,
                        int rowdim, double *I, int centerLo, int centerHi,
                        OracleStats *stats);

/* Records every block in the reference's callback order (centre C, atom A,
 * atom B >= A, shell s1, shell s2, type 1 then type 2).  meta gets 8 ints per
 * block: A, s1, la, B, s2, lb, C, type.  data gets the IJK(la) x IJK(lb)
 * row-major blocks back to back.  Returns as oracle_getIntegrals, or -2 when
 * the output buffers are too small. */
int oracle_blocks(int nrAtoms, const double *geometry,
                  const int *shellsECP, const int *KECP, const int *lECP,
                  const double *nECP, const double *dECP, const double *aECP,
                  const int *shellsBS, const int *lBS, const int *KBS,
                  const double *dBS, const double *aBS,
                  int largeGridOrder, double tolerance, double accuracy,
                  int centerLo, int centerHi,
                  int maxBlocks, int *meta, long long maxData, double *data,
                  int *nBlocks, long long *nData, OracleStats *stats);

/* getIntegrals over nThreads POSIX threads: ECP centres are dealt round-robin
 * to threads, each thread owns a private matrix, and the partial matrices are
 * summed into I at the end.  Used as the all-core CPU baseline. */
/* As oracle_blocks, plus alternative blocks: for every block whose
 * quadratures took a convergence decision within rounding noise (the test's
 * two sides closer than kappa * 2^-53 * sum |w f| allows), the block
 * recomputed with chosen such decisions inverted, recorded with the same
 * meta rows into altMeta / altData (several per block possible).  scale (one
 * per block, or NULL): the largest element of the block evaluated over
 * absolute values (the angular contractions and the shift onto A and B with
 * |factor| and |term|), which sets the size of any FP64 evaluation's rounding. */
int oracle_blocks_alt(int nrAtoms, const double *geometry,
                      const int *shellsECP, const int *KECP, const int *lECP,
                      const double *nECP, const double *dECP, const double *aECP,
                      const int *shellsBS, const int *lBS, const int *KBS,
                      const double *dBS, const double *aBS,
                      int largeGridOrder, double tolerance, double accuracy,
                      int centerLo, int centerHi, double kappa, int maxBlocks, int *meta,
                      long long maxData, double *data, double *scale, int *nBlocks,
                      long long *nData, int maxAlt, int *altMeta, long long maxAltData, double *altData,
                      int *nAlt, long long *nAltData, OracleStats *stats);

int oracle_getIntegrals_mt(int nrAtoms, const double *geometry,
                           const int *shellsECP, const int *KECP, const int *lECP,
                           const double *nECP, const double *dECP, const double *aECP,
                           const int *shellsBS, const int *lBS, const int *KBS,
                           const double *dBS, const double *aBS,
                           int largeGridOrder, double tolerance, double accuracy,
                           int rowdim, double *I, int nThreads, OracleStats *stats);

/* Table probes used by the unit tests (each writes into caller memory). */
int oracle_grid(int which, int maxPoints, double *x, double *w); /* 0 = PS93+KK, 1 = PSM92 */
int oracle_bessel(int lmax, double z, int tabLmax, double accuracy, double *K);
int oracle_rsh(int lmax, double theta, double phi, double *out);

#ifdef __cplusplus
}
#endif
#endif
