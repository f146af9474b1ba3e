/*
 * ref_driver.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Thin driver compiled together with the unmodified libECP sources
 * (the .c files under src/ of chrr/libECP) into oracle/_ref/libecp_ref.so by oracle/Makefile.
 * It calls the reference's own public API -- libECP_init /
 * calculateECPIntegrals / libECP_free (src/libecp.h:15-29) -- with a callback
 * that records every block the reference hands out at src/libecp.c:372, in
 * the order they arrive.  The callback's argument order follows the call site
 * (A, s1, la, shifta, B, s2, lb, shiftb, C, I, p), which is also how
 * src/getIntegrals.c:23-25 implements it.
 *
 * The reference calls the callback twice per (shell pair, ECP centre): first
 * with the type-1 (local) block, then with the type-2 (semi-local) block
 * (src/libecp.c:332-374).  ref_blocks() tags them 1 and 2 in that order.
 */
#include <stdlib.h>
#include <string.h>
#include "libecp.h"
#include "getIntegrals.h"

#define IJK(l) (((l) + 1) * ((l) + 2) / 2)

typedef struct {
  int maxBlocks, nBlocks;
  int *meta;          /* 8 ints per block: A, s1, la, B, s2, lb, C, type */
  long long maxData, nData;
  double *data;
  int overflow;
  int lastKey[5];
  int lastType;
} Recorder;

static void record_block(int A, int sa, int la, int shifta, int B, int sb,
                         int lb, int shiftb, int C, double *I, void *p) {
  Recorder *r = (Recorder *)p;
  int key[5] = {A, sa, B, sb, C};
  int type = 1;
  long long n = (long long)IJK(la) * IJK(lb);
  (void)shifta; (void)shiftb;
  if (r->nBlocks > 0 && r->lastType == 1 && memcmp(key, r->lastKey, sizeof key) == 0)
    type = 2;
  memcpy(r->lastKey, key, sizeof key);
  r->lastType = type;
  if (r->nBlocks >= r->maxBlocks || r->nData + n > r->maxData) {
    r->overflow = 1;
    return;
  }
  int *m = r->meta + 8 * r->nBlocks;
  m[0] = A; m[1] = sa; m[2] = la; m[3] = B; m[4] = sb; m[5] = lb; m[6] = C; m[7] = type;
  memcpy(r->data + r->nData, I, n * sizeof(double));
  r->nData += n;
  r->nBlocks++;
}

/* Runs the reference on one system and records all blocks.
 * Argument meaning follows getIntegrals (src/getIntegrals.h:7-13): KECP is the
 * number of terms per ECP shell, lECP the angular momentum of each ECP shell.
 * Returns: 0 ok, -1 init failed (NULL handle), -2 output buffers too small,
 * otherwise the nonzero status of calculateECPIntegrals. */
int ref_blocks(int nrAtoms, double *geometry, int *shellsECP, int *KECP,
               int *lECP, double *nECP, double *dECP, double *aECP,
               int *shellsBS, int *lBS, int *KBS, double *dBS, double *aBS,
               int largeGridOrder, double tolerance, double accuracy,
               int maxBlocks, int *meta, long long maxData, double *data,
               int *nBlocks, long long *nData) {
  Recorder r;
  memset(&r, 0, sizeof r);
  r.maxBlocks = maxBlocks; r.meta = meta; r.maxData = maxData; r.data = data;
  /* libECP_init's definition reads (shellsECP, lECP, KECP), src/libecp.c:55 */
  libECPHandle *h = libECP_init(nrAtoms, geometry, shellsECP, lECP, KECP, nECP,
                                dECP, aECP, shellsBS, lBS, KBS, dBS, aBS, 0, -1,
                                NULL, largeGridOrder, tolerance, accuracy);
  if (h == NULL) return -1;
  int st = calculateECPIntegrals(h, record_block, &r);
  libECP_free(h);
  *nBlocks = r.nBlocks;
  *nData = r.nData;
  if (r.overflow) return -2;
  return st;
}

/* ---- derivative blocks (libECP_init's n = 1, 2) ----
 * The reference hands out, per (shell pair, centre) and derivative shift
 * (shifta, shiftb), a type-1 and a type-2 block of the shifted shells
 * (src/libecp.c:322-374); for n = 2 the shifts (+1, 0) and (0, +1) keep the
 * unshifted l in the block (src/libecp.c:356-362).  Recorded with 10 ints per
 * block: A, s1, la, shifta, B, s2, lb, shiftb, C, type. */
typedef struct {
  int n, maxBlocks, nBlocks;
  int *meta;
  long long maxData, nData;
  double *data;
  int overflow;
  int lastKey[7];
  int lastType;
} DerivRecorder;

static void record_deriv(int A, int sa, int la, int shifta, int B, int sb,
                         int lb, int shiftb, int C, double *I, void *p) {
  DerivRecorder *r = (DerivRecorder *)p;
  int key[7] = {A, sa, B, sb, C, shifta, shiftb};
  int type = 1, lpa = la + shifta, lpb = lb + shiftb;
  if (r->n == 2 && shifta == 1 && shiftb == 0) lpa = la;
  if (r->n == 2 && shifta == 0 && shiftb == 1) lpb = lb;
  long long n = (long long)IJK(lpa) * IJK(lpb);
  if (r->nBlocks > 0 && r->lastType == 1 && memcmp(key, r->lastKey, sizeof key) == 0)
    type = 2;
  memcpy(r->lastKey, key, sizeof key);
  r->lastType = type;
  if (r->nBlocks >= r->maxBlocks || r->nData + n > r->maxData) {
    r->overflow = 1;
    return;
  }
  int *m = r->meta + 10 * r->nBlocks;
  m[0] = A; m[1] = sa; m[2] = la; m[3] = shifta; m[4] = B; m[5] = sb; m[6] = lb; m[7] = shiftb;
  m[8] = C; m[9] = type;
  memcpy(r->data + r->nData, I, n * sizeof(double));
  r->nData += n;
  r->nBlocks++;
}

int ref_blocks_deriv(int nrAtoms, double *geometry, int *shellsECP, int *KECP,
                     int *lECP, double *nECP, double *dECP, double *aECP,
                     int *shellsBS, int *lBS, int *KBS, double *dBS, double *aBS,
                     int largeGridOrder, double tolerance, double accuracy, int n,
                     int maxBlocks, int *meta, long long maxData, double *data,
                     int *nBlocks, long long *nData) {
  DerivRecorder r;
  memset(&r, 0, sizeof r);
  r.n = n; r.maxBlocks = maxBlocks; r.meta = meta; r.maxData = maxData; r.data = data;
  libECPHandle *h = libECP_init(nrAtoms, geometry, shellsECP, lECP, KECP, nECP,
                                dECP, aECP, shellsBS, lBS, KBS, dBS, aBS, n, -1,
                                NULL, largeGridOrder, tolerance, accuracy);
  if (h == NULL) return -1;
  int st = calculateECPIntegrals(h, record_deriv, &r);
  libECP_free(h);
  *nBlocks = r.nBlocks;
  *nData = r.nData;
  if (r.overflow) return -2;
  return st;
}

/* The blocks of derivative order 0 in a caller's Cartesian order
 * (libECP_init's lmax and shellOrdering, src/libecp.c:159-165); recorded as
 * ref_blocks does. */
int ref_blocks_ordered(int nrAtoms, double *geometry, int *shellsECP, int *KECP,
                       int *lECP, double *nECP, double *dECP, double *aECP,
                       int *shellsBS, int *lBS, int *KBS, double *dBS, double *aBS,
                       int largeGridOrder, double tolerance, double accuracy,
                       int lmax, int *ordering,
                       int maxBlocks, int *meta, long long maxData, double *data,
                       int *nBlocks, long long *nData) {
  Recorder r;
  memset(&r, 0, sizeof r);
  r.maxBlocks = maxBlocks; r.meta = meta; r.maxData = maxData; r.data = data;
  libECPHandle *h = libECP_init(nrAtoms, geometry, shellsECP, lECP, KECP, nECP,
                                dECP, aECP, shellsBS, lBS, KBS, dBS, aBS, 0, lmax,
                                ordering, largeGridOrder, tolerance, accuracy);
  if (h == NULL) return -1;
  int st = calculateECPIntegrals(h, record_block, &r);
  libECP_free(h);
  *nBlocks = r.nBlocks;
  *nData = r.nData;
  if (r.overflow) return -2;
  return st;
}

