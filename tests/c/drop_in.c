/* A C host program that uses libecp_gb300 exactly as a caller of the
 * reference's library would (getIntegrals.h, libecp.h): one getIntegrals
 * call and one libECP_init / calculateECPIntegrals / libECP_free pass over a
 * small system, printed as "M i j value" (matrix) and "B A s1 la B s2 lb C
 * first-value" (callback blocks) lines.  Test infrastructure: built and run
 * by tests/test_c_drop_in.py. */
#include <stdio.h>
#include <stdlib.h>

#include "getIntegrals.h"
#include "libecp.h"

static void record(int A, int sa, int la, int shifta, int B, int sb, int lb, int shiftb, int C,
                   double *I, void *p) {
  (void)shifta; (void)shiftb; (void)p;
  printf("B %d %d %d %d %d %d %d %.17g\n", A, sa, la, B, sb, lb, C, I[0]);
}

int main(void) {
  /* one ECP centre (channels l = 0, 1 and the local l = 2) at the origin,
   * two atoms with an s and a p shell */
  double geometry[9] = {0.0, 0.0, 0.0, 0.9, -0.4, 0.3, -0.7, 0.5, 0.8};
  int shellsECP[3] = {3, 0, 0};
  int KECP[3] = {2, 1, 2};
  int lECP[3] = {0, 1, 2};
  double nECP[5] = {2.0, 1.0, 2.0, 2.0, 0.0};
  double dECP[5] = {3.0, -1.2, -2.0, 1.5, 0.4};
  double aECP[5] = {1.3, 0.4, 0.7, 2.1, 0.9};
  int shellsBS[3] = {0, 2, 2};
  int lBS[4] = {0, 1, 0, 1};
  int KBS[4] = {2, 1, 1, 2};
  double dBS[6] = {0.6, 0.4, 0.9, 0.7, 0.5, 0.8};
  double aBS[6] = {1.7, 0.3, 0.8, 1.1, 2.4, 0.6};
  const int dim = 1 + 3 + 1 + 3;
  double *I = calloc(dim * dim, sizeof(double));
  int rc = getIntegrals(3, geometry, shellsECP, KECP, lECP, nECP, dECP, aECP, shellsBS, lBS, KBS, dBS,
                        aBS, 1024, 1.0E-12, 1.0E-14, dim, I);
  printf("RC %d\n", rc);
  for (int i = 0; i < dim; i++)
    for (int j = i; j < dim; j++) printf("M %d %d %.17g\n", i, j, I[i * dim + j]);
  /* the handle interface reads (shellsECP, lECP, KECP), src/libecp.c:55 */
  libECPHandle *h = libECP_init(3, geometry, shellsECP, lECP, KECP, nECP, dECP, aECP, shellsBS, lBS,
                                KBS, dBS, aBS, 0, -1, NULL, 1024, 1.0E-12, 1.0E-14);
  if (!h) {
    printf("INIT NULL\n");
    return 1;
  }
  printf("CB %d\n", calculateECPIntegrals(h, record, NULL));
  libECP_free(h);
  free(I);
  return 0;
}
