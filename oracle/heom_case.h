/* Test infrastructure: the oracle's flat description of one HEOM instance.
 *
 * Shared by the CPU restatement (oracle/heom_oracle.cpp) and the harness that
 * compiles the reference's own model/integrator code (oracle/refharness/).
 * Every complex number is two doubles (re, im); matrices are row-major.
 * The fields are the reference's public parameter members (qme_base.h:32-67,
 * heom.h:44-50); per-bath arrays are concatenated bath after bath. */
#ifndef HEOM_CASE_H
#define HEOM_CASE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct heom_case {
  int n_level;           /* n: Hilbert-space dimension                      */
  int n_noise;           /* U: number of baths                              */
  int max_depth;         /* N: hierarchy depth                              */
  const double* H;       /* n*n complex                                     */
  const double* V;       /* U*n*n complex                                   */
  const int* len_gamma;  /* U                                               */
  const double* gamma;   /* sum_u len_u^2 complex                           */
  const double* phi_0;   /* sum_u len_u complex                             */
  const double* sigma;   /* sum_u len_u complex                             */
  const double* S;       /* sum_u len_u^2 complex                           */
  const double* A;       /* sum_u len_u^2 complex                           */
  const double* s_delta; /* U complex                                       */
  int sqrt_normalization; /* 1: LIBHEOM_SQRT_NORMALIZATION (heom_hilb.h:140-196) */
  int col_major;          /* 1: the `col_major` order: each ADO stored column-major */
  /* hrchy_filter of alloc_hrchy_space (hrchy_space.h:29-36) with filter_flag
   * true when non-null: nonzero keeps the candidate multi-index */
  int (*hrchy_filter)(const int* index, int n_dim, int depth, void* user);
  void* filter_user;
} heom_case;

/* form: 0 = heom_hilb, 1 = heom_liou (CSR superoperators), 2 = heom_ado.
 * solver: 0 = rk4, 1 = lsrk4, 2 = rkdp. */

#ifdef __cplusplus
}
#endif
#endif
