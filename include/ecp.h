/*
 * ecp.h -- ECP model structures of the drop-in library.
 *
 * Same layout and functions as chrr/libECP's src/ecp.h:9-41 (the structures
 * are part of the interface callers compile against).  An ECP is a list of
 * Gaussian terms d * r^n * exp(-a r^2), each tagged with its channel l;
 * channel L is the local part, channels l < L the semi-local ones.
 */
#ifndef ECP_H
#define ECP_H 1

#ifdef __cplusplus
extern "C" {
#endif

typedef struct _ECPGauss ECPGauss;
typedef struct _ECP ECP;

struct _ECPGauss {
  int l;
  double a, d, n;
};

struct _ECP {
  ECPGauss *U_l; /* Gaussian terms                 */
  int N;         /* number of terms                */
  int L;         /* highest channel (local part)   */
};

/* Allocates an ECP with N terms, all tagged l = -1 (src/ecp.c:28).  Free with ECP_free. */
ECP *newECP(const int L, const int N);

/* 0 if the terms are sorted by l and every l lies in [0, L], else 1 (src/ecp.c:9-26). */
int checkECP(const ECP *U);

/* Number of terms with channel l; *U_l receives a malloc'ed copy of them
 * (declared at src/ecp.h:34; the reference never defines it). */
int getECP(const ECP *U, const int l, ECPGauss **U_l);

/* U_l(r) = sum over terms with channel l of d r^n exp(-a r^2) (src/ecp.c:42-60). */
double evalECP(const ECP *U, const int l, const double r);

void ECP_free(ECP *E);

#ifdef __cplusplus
}
#endif
#endif /* ECP_H */
