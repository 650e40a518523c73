/*
 * pn_oracle.h -- CPU restatement of the reference PN march (test infrastructure only).
 * See pn_oracle.c for what is restated and from where.
 */
#ifndef PN_ORACLE_H
#define PN_ORACLE_H

#include <stdint.h>

#include "../include/pnepma.h"

#define ORA_MAXN 15
#define ORA_MAXM 64     /* moments per class at ORA_MAXN: N_eee(15) = 36 */
#define ORA_MAXE 8
#define ORA_MAXR 16

#ifdef __cplusplus
extern "C" {
#endif

/* 1 when built with OpenMP; ora_set_threads sets the host threads of one solve (returns the
   count in effect: 1 without OpenMP) */
int ora_openmp(void);
int ora_set_threads(int n);
int64_t ora_state_size(const pn_desc* d);
int64_t ora_rho_size(const pn_desc* d);
/* calc_intensities; tape (optional) receives the n_steps + 1 states */
int ora_forward(const pn_desc* d, const double* rho, const double* noa, const double* acs,
                double* intensities, double* tape);
/* forward (intensities, optional) + calc_intensities_pullback up to the material pullbacks */
int ora_adjoint(const pn_desc* d, const double* rho, const double* noa, const double* acs,
                const double* Ibar, double* intensities, double* rho_bar, double* noa_bar,
                double* acs_bar);
int ora_generation_field(const pn_desc* d, const double* rho, double* field);
/* one forward energy step of `state` in place */
int ora_step(const pn_desc* d, const double* rho, double* state, int step);
/* many independent forward+adjoint solves on `threads` host threads (CPU baseline) */
int ora_solve_many(const pn_desc* const* d, const double* const* rho, const double* const* noa,
                   const double* const* acs, const double* const* Ibar, double* const* intensities,
                   double* const* rho_bar, double* const* noa_bar, double* const* acs_bar, int n,
                   int threads);

#ifdef __cplusplus
}
#endif
#endif
