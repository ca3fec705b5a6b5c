/*
 * oracle/port/port.h -- C API of the CPU restatement of bmagwa's sampler.
 *
 * ORACLE / TEST INFRASTRUCTURE.  This is the oracle the GPU path is compared
 * against and the CPU baseline bench.py times; it is never linked into, or
 * called by, the product.  It restates the reference algorithm
 * (src/sampler.hpp, src/sampler.cpp, src/model.hpp, src/prior.*, src/data*.cpp,
 * src/precomputed_snp_covariances.hpp, src/discrete_distribution.hpp) in the
 * reference's floating-point operation order, on the random stream of
 * include/bmg_rng.h, so its traces equal those of the reference compiled in
 * oracle/_ref bit for bit.  Scope: PMV sampler (moves 0-3), delayed rejection
 * off, all effect types, missing genotypes, individual or shared tau2.
 */
#ifndef BMG_ORACLE_PORT_H_
#define BMG_ORACLE_PORT_H_

#include <stddef.h>
#include <stdint.h>
#include "bmg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bmgport bmgport;

/* packed: m_g rows of ceil(n/4) bytes (PLINK SNP-major payload); y: n values;
 * e: n x m_e covariates without the constant (column-major) or NULL. */
int bmgport_create(const bmg_options* opt, const uint8_t* packed, const double* y,
                   const double* e, bmgport** out, char* err, size_t err_len);
/* advance every chain n_iter iterations (threads = min(chains, n_threads)) */
int bmgport_run(bmgport* P, uint64_t n_iter, uint32_t n_threads,
                const bmg_trace_sink* sink);
/* RB scan of one chain against y - y_hat of its current model */
int bmgport_scan(bmgport* P, uint32_t chain, double* p_r, double* p_r_types);
int bmgport_scan_logodds(bmgport* P, uint32_t chain, double* logodds);
int bmgport_schur(bmgport* P, uint32_t chain, double* dlml, double* itv);
/* RB scan of one chain against y - y_hat with sigma2 replaced (known-answer tests) */
int bmgport_scan_yhat(bmgport* P, uint32_t chain, const double* y_hat, double sigma2,
                      double* p_r, double* p_r_types);
int bmgport_scan_yhat_logodds(bmgport* P, uint32_t chain, const double* y_hat, double sigma2, double* logodds);
int bmgport_get_state(bmgport* P, uint32_t chain, bmg_chain_state* st,
                      uint32_t* loci, uint8_t* type_inds, uint32_t cap);
/* the prior's shared 1/(tau2 alpha^2) per term type (A, H, D, R) */
int bmgport_get_inv_tau2_alpha2(bmgport* P, uint32_t chain, double* out4);
int bmgport_get_rao(bmgport* P, uint32_t chain, double* p_rao, double* p_rao_types);
/* the adaptive proposal p_proposal (src/sampler.hpp:363-383) */
int bmgport_get_proposal(bmgport* P, uint32_t chain, double* p_prop, double* p_prop_types);
/* p_r of the last in-loop RB scan (src/sampler.cpp:731-757) */
int bmgport_get_last_scan(bmgport* P, uint32_t chain, double* p_r, double* p_r_types);
int bmgport_get_precomputed(bmgport* P, double* xx, uint32_t* offset);
/* var_x, mean_x, var_y, yy of the loaded data (src/data.hpp:66-71) */
int bmgport_get_data_stats(bmgport* P, double* out4);
/* decoded genotype column of one SNP for a term type (missing -> -1) */
int bmgport_get_genotypes(bmgport* P, uint32_t type, uint64_t snp, double* out);
/* LML after each add_term of a fresh model (src/model.hpp:239-268) */
int bmgport_model_lml(bmgport* P, uint32_t n_add, const uint32_t* snps,
                      const uint8_t* t_inds, const double* inv_tau2_alpha2,
                      double* lml_after_each);
/* exhaustive model set of the last n_terms - const_loci terms (2^m log
   probabilities) and the same probabilities from models built directly
   (src/sampler.cpp:882-978, src/tests/model_tests.hpp:92-235) */
int bmgport_exh_modelset(bmgport* P, uint32_t n_terms, const uint32_t* snps,
                         const uint8_t* t_inds, const double* inv_tau2_alpha2,
                         uint32_t const_loci, double* exh_out, double* direct_out);
/* log proposal probabilities of the 2^n_inds sub-models of a
   delayed-rejection move (src/sampler.cpp:980-1049); out is added to */
int bmgport_exh_proposal_probs(int use_types, int n_inds, const uint8_t* bit_to_normalized_order,
                               const double* q_add, const double* q_rem, double z_add, double z_rem,
                               uint64_t const_loci, uint64_t m_g, const double* log_q_add_types,
                               double* out);
/* LML after n_add add_term calls and one remove_term (src/model.hpp:270-312) */
int bmgport_model_lml_remove(bmgport* P, uint32_t n_add, const uint32_t* snps, const uint8_t* t_inds,
                             const double* inv_tau2_alpha2, uint32_t rem, double* lml);
/* the proposal tree alone: zero/restore ops, node values, total, draw counts
   (src/discrete_distribution.hpp:64-330) */
int bmgport_dd_exercise(const double* w, uint64_t n, const int64_t* ops, uint64_t n_ops, uint32_t seed,
                        uint64_t n_samples, double* values_out, double* total_out, uint64_t* counts_out);
/* n_reps imputations of one SNP's missing calls; the count of each value
   imputed for its first missing call, the corrected precomputed row and the
   four codings after the last draw (src/data_model.cpp:90-167) */
int bmgport_missing_step(bmgport* P, uint32_t chain, uint64_t snp, uint64_t n_reps, double* xx_out,
                         double* geno_out, uint64_t* counts);
/* n_samples draws of (sigma2, beta) given a model of n_add terms
   (src/model.hpp:326-342); beta_out rows of blen_cap values */
int bmgport_sample_beta_sigma2(bmgport* P, uint32_t n_add, const uint32_t* snps, const uint8_t* t_inds,
                               const double* inv_tau2_alpha2, uint32_t seed, uint64_t n_samples, double* s2_out,
                               double* beta_out, uint32_t blen_cap, uint32_t* blen);
/* log model prior of Ns and its changes on add / remove (type ta, nl loci)
   and on a type switch ta -> tr (src/prior.hpp:144-183) */
int bmgport_prior_terms(bmgport* P, const int32_t* Ns, int32_t nl, int32_t ta, int32_t tr, double* out);
void bmgport_destroy(bmgport* P);

#ifdef __cplusplus
}
#endif

#endif
