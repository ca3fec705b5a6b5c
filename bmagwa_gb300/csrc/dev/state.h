// Device-resident data layout of libbmg (shared by host and device code).
//
// HBM layout (one context):
//   geno      m_g rows of `gs` bytes: PLINK 2-bit codes, 4 individuals per
//             byte, rows padded to a multiple of 16 bytes (64 individuals);
//             padding codes are 00 and every padded individual carries a zero
//             residual, so it adds nothing to any product.
//   cnt       per SNP: counts of genotype 1 and 2 (missing codes rejected).
//   pre       per SNP: the reference's precomputed sums and centred second
//             moments (src/precomputed_snp_covariances.hpp:42-84 layout).
//   inorder   heap node -> in-order rank of the reference's proposal tree
//             (src/discrete_distribution.hpp:217-261) and its inverse.
//   per chain: two models (current, proposed), the dynamic sampler state,
//             proposal arrays of m_g doubles, a prefix array of m_g+1
//             doubles, a model-membership bitmap and model index map.
#ifndef BMG_DEV_STATE_H_
#define BMG_DEV_STATE_H_

#include <stdint.h>

#include "bmg_rng.h"

#define BMG_MOVE_THREADS 256
#define BMG_PEND_MAX 64          /* pending zero/unzero flips of dd_add */
#define BMG_PEND_REBUILD 8       /* more pending flips at an RB step: rebuild the prefix */
#define BMG_REBUILD_TILE 4096    /* in-order positions per CTA of the prefix rebuild */
#define BMG_MAX_MS 255
#define BMG_REMSET_MAX 1280      /* in-model SNPs + moved SNPs for dd_rem */
#define BMG_MAX_COV 31            /* covariates besides the constant */
#define BMG_DR_MAX 16            /* delayed rejection: largest move whose 2^m sub-models are enumerated */

// One model (bmagwa::Model, src/model.hpp:394-423) of one chain.
// Matrices are column-major with leading dimension km (max_model_size).
struct DevModel {
  int k;          // loci in the model
  int xcols;      // columns of X (covariates incl. constant + terms)
  int llen;       // active order of l
  int vlen;       // active length of v
  int blen;       // active length of beta
  int Ns[5];
  int mu_beta_computed;
  int pad_;
  double sigma2, syx, ldq, ldqx, ll;
  // arrays (device pointers into the chain's arena)
  double* xx;     // km x km upper
  double* l;      // km x km upper Cholesky factor
  double* xy;     // km
  double* v;
  double* inv;    // inv_tau2_alpha2 per column
  double* beta;
  double* mu_beta;
  uint32_t* loci;       // km
  uint8_t* type_inds;   // km
  uint32_t* x_ind1;
  uint32_t* x_ind2;
  uint32_t* xc_snp;     // x_ind_to_g_ind
  int32_t* xc_type;     // x_types (4 = covariate)
};

// Dynamic per-chain sampler state (bmagwa::Sampler members that change).
struct DevChain {
  bmg_rng_t rng;
  uint64_t n_iter;
  uint64_t n_accepted;
  uint64_t n_rao_burnin;     // remaining
  uint64_t p_proposal_n;
  int64_t p_rao_n;
  uint64_t n_moves[7];
  uint64_t n_acpt[7];
  uint64_t n_lik_add, n_lik_rem, n_lik_full;
  double alpha, alpha2;       // Prior::alpha_ / alpha2_
  double inv_t2a2[4];         // Prior::inv_tau2_alpha2
  double p_move_size;
  double k_move_size;
  double pves[3];
  double yhat_absmax;         // max |y_hat| after the last PVE pass
  int started;
  int movesize;
  int error;                  // 0 = fine; see BMG_DERR_*
  int rb_pending;             // an RB scan must follow this launch
  // dd_add prefix bookkeeping
  int64_t cadd_total;         // prefix[m_g] at the last rebuild
  int n_pend;
  int rebuild;                // proposal weights changed: rebuild prefix
  int pend_snp[BMG_PEND_MAX];
  // trace cursor (reset by the host per chunk)
  uint32_t tr_iter;
  uint32_t tr_thin;
  uint32_t tr_loci;
  uint32_t tr_beta;
  uint32_t tr_log;
};

// one _log.txt line (src/sampler.cpp:813-833): iter, n_accepted, n_acpt[1],
// n_moves[1], n_acpt[2], n_moves[2], p_move_size, model size, log p, pve[3], sigma2
#define BMG_LOGREC 13

// Device error codes (DevChain::error)
#define BMG_DERR_NONE 0
#define BMG_DERR_CAPACITY 1      // model larger than max_model_size
#define BMG_DERR_NAN 2           // NaN where the reference throws
#define BMG_DERR_RNG 3           // gamma sampler ran out of attempts
#define BMG_DERR_PEND 4          // pending proposal list overflow
#define BMG_DERR_TRACE 5         // trace buffer overflow
#define BMG_DERR_REMSET 6
#define BMG_DERR_START 7         // non-finite likelihood at start
#define BMG_DERR_TIMEOUT 8       // a bounded device wait gave up

// Parameters the move kernel hands to the RB scan epilogue, per chain.
struct RbParams {
  double inv_2s2;           // 1 / (2 sigma2)
  double mr;                // mean residual
  double scale;             // 2^-s of the fixed-point residual
  double itv[4];            // inv_tau2_alpha2 per term (shared tau2)
  double nlog_itv[4];       // -log(itv[t]), once per chain
  double cadd[4];           // lmp_add[t] - nlog_itv[t] / 2: the odds' constant
  float scale_f;            // scale as FP32 (a power of two)
  float mr_df[2], i2s_df[2];          // mr and inv_2s2 as FP32 pairs (hi, lo)
  float itv_df[4][2], cadd_df[4][2];  // itv[t] and cadd[t] as FP32 pairs
  double lmp_add[5];
  double lmp_rem[5][5];
  double rao_iz1, rao_z2;   // running mean of p_rao: z2 old + p / z1, 1/z1 kept
  double prop_iz1, prop_z2; // running mean of p_proposal, the same form
  double alpha2;            // Prior::alpha2_ for per-SNP tau2 draws
  uint64_t rng_slot;        // first stream slot of the per-SNP tau2 draws
  uint32_t key0, key1;      // chain stream key
  int do_scan;              // compute p_r at all this step
  int acc_rao;              // n_rao_burnin <= 0: accumulate p_rao
  uint64_t miss_slot;       // first stream slot of the imputation of the missing calls outside the model
  int n_inm;                // in-model SNPs listed in DevConst::miss_inm
  int adapt;                // update p_proposal and the proposal weights
};

// Scan corrections of one (chain, SNP with missing calls) at an RB step: the
// SNP's missing calls enter the scan's products as 0; these add what their
// imputed values contribute (src/data_model.cpp:30-72, 105-167).
#define BMG_MAX_OFFSET 9
struct MissCorr {
  long long dxr[4];              // sum over the missing calls of x_t(value) R_i (fixed point)
  double pre[BMG_MAX_OFFSET];    // the precomputed values as DataModel::update_prexx_cov corrects them
  int dsum[4];                   // sum of x_t(value)
  int dcross[4][4];              // sum of x_t(value) x_u(value)
};

// Trace buffers of one chunk (device), per chain.
struct DevTrace {
  uint8_t* jump;      // chains x iters
  uint8_t* mtype;
  uint8_t* msize;
  uint32_t* msz;      // chains x thin_cap
  uint32_t* loci;     // chains x loci_cap
  uint8_t* types;     // chains x loci_cap
  double* ll;         // chains x thin_cap
  double* lp;
  double* s2;
  double* alpha;
  double* pve;        // chains x thin_cap x 3
  double* beta;       // chains x beta_cap
  double* logrec;     // chains x log_cap x BMG_LOGREC doubles (the _log.txt lines)
  uint32_t iter_cap, thin_cap, loci_cap, beta_cap, log_cap;
};

// Read-only context constants.
// The sample a chain is fitted to: one phenotype and the individuals it has
// a value for.  All chains of a context share one record unless the context
// holds several phenotypes (then chain c uses record c).  Counts, sums and
// the fixed-point phenotype are over the sample only; the phenotype is zero
// outside it, so products with it need no mask.
struct DevPheno {
  double n;              // individuals in the sample
  double n_plus_nu, minus_n_plus_nu_2, nus2_plus_yy, rng_nu;
  double nus2_tau2[4];   // nu_t s2_t of the term precisions' prior
  double y_absmax;
  int32_t sy;            // fixed-point exponent of y
  const double* y;       // n entries (0 outside the sample)
  const int64_t* yint;   // n entries, y 2^sy rounded
  const uint64_t* mask2; // gs / 8 words: 01 in the 2-bit slot of each individual in the sample; null: all
  const int32_t* cnt;    // p x 2: #het, #hom-alt within the sample
  const double* pre;     // p x offset: the precomputed sums within the sample
  const float4* pre_f;   // one-type scans: {sum x, pre1 hi, pre1 lo, 0} per SNP, else null
  const int64_t* gsum;   // p x nv x 2 fixed-point sums of y and covariates, or null (X'y from the codes)
};

// The learned part of the add proposal (no reference counterpart): a
// 16 -> 128 -> 128 -> 1 MLP shared by the chains, its per-chain candidate
// tables and the buffers of its features.  FP32 master parameters in one
// array (W1 128x16, b1, W2 128x128, b2, w3, b3), bf16 copies of W1 and W2 for
// the tensor-core forward pass.
#define MLP_F 16
#define MLP_H 128
#define MLP_OW1 0
#define MLP_OB1 (MLP_OW1 + MLP_H * MLP_F)
#define MLP_OW2 (MLP_OB1 + MLP_H)
#define MLP_OB2 (MLP_OW2 + MLP_H * MLP_H)
#define MLP_OW3 (MLP_OB2 + MLP_H)
#define MLP_OB3 (MLP_OW3 + MLP_H)
#define MLP_NPAR (MLP_OB3 + 1)
struct DevLearned {
  int on;               // BMG_PROPOSAL_LEARNED
  double mix;           // weight of the MLP part
  uint32_t topk;        // candidate table size per chain
  uint32_t* t_snp;      // chains x topk: candidates in ascending SNP order
  double* t_s;          // chains x topk: their weights (predicted inclusion probability)
  double* t_sum;        // chains: sum of the weights
  uint32_t* t_n;        // chains: candidates in the table
  float* maxcorr;       // chains x p: max |corr| to the model's SNPs within the LD window
  float* logit;         // chains x p: MLP output of the last refresh
  float* theta;         // MLP_NPAR parameters
  float* grad;          // MLP_NPAR gradient accumulator
  float* adam_m;
  float* adam_v;
  uint16_t* w1b;        // bf16 W1 (128 x 16)
  uint16_t* w2b;        // bf16 W2 (128 x 128)
};

struct DevConst {
  // sizes
  uint64_t n;           // individuals
  uint64_t p;           // SNPs (m_g)
  uint32_t gs;          // bytes per genotype row (multiple of 16)
  uint32_t nw;          // 32-bit words per genotype row (gs / 4)
  uint32_t m_e;         // covariate columns incl. the constant
  uint32_t km;          // max_model_size
  uint32_t n_chains;
  uint32_t n_types;
  int32_t types[5];
  int32_t allow_types[5];
  int32_t allow_terms[4];
  int32_t offset;       // per-SNP doubles of `pre`
  int32_t offset_type[4];
  uint32_t n_terms;     // allowed terms (rows per SNP in the scan)
  int32_t term_of[4];   // scan row r -> term type
  // sampler options
  uint64_t n_rao, thin, n_sample_tau2, verbosity;
  uint32_t max_move_size;       // already min(m_g, 255, option)
  uint32_t max_nbh;
  double p_move_size_nbs, p_move_size_nbc;
  int32_t adapt_p_move_size;
  double acpt_goal;
  int32_t adaptation, flat_proposal_dist, save_beta;
  double q_add_min, q_rem_min;
  // prior constants (per context; sigma2 terms per phenotype below)
  double n_plus_nu, minus_n_plus_nu_2, nus2_plus_yy;
  double mu_alpha;
  int32_t use_individual_tau2;
  double g_a, g_b;
  double types_prior[5], types_prior_sum;
  double nu_tau2[4], s2_tau2[4], nus2_tau2[4];
  double rng_nu;        // n + nu_sigma2 (src/sampler.hpp:127)
  // Host-computed prior tables (index = a count 0..km+1), evaluated with the
  // reference's own expressions (src/prior.hpp:144-183) by the host libm:
  //   add_a[nl] = log(g_a + nl) - log(g_b + m_g - nl - 1)
  //   rem_a[nl] = log(g_b + m_g - nl) - log(g_a + nl - 1)
  //   lt[t][k] = log(tp[t] + k),   ltm1[t][k] = log(tp[t] + k - 1)
  //   ls[k] = log(tps + k),        lsm1[k] = log(tps + k - 1)
  //   lgt[t][k] = lgamma(tp[t] + k), lga[k] = lgamma(g_a + k),
  //   lgb[k] = lgamma(g_b + m_g - k), lgs[k] = lgamma(tps + k)
  // Layout: one array `tab`, each table tw = km + 2 entries; typed tables
  // hold 5 rows.
  const double* tab;
  uint32_t tw;
  int32_t qs;           // fixed-point exponent of the dd_add weights
  // move-size adaptation (src/sampler.hpp:1728-1769): the 50 grid values of p
  // the reference visits (p = 0.01; p += 0.98 / 49) and pow(1 - p, max_ms) for
  // each grid value [0..49] and for the initial p_move_size [50], by the host libm
  const double* ms_grid;
  const double* ms_pow;
  double ms_init;
  // data
  const uint8_t* geno;
  const int32_t* cnt;   // p x 2
  const double* pre;    // p x offset
  const double* lvar;   // p x n_terms: log of the centred second moment
  const int32_t* pos;   // heap node -> in-order rank
  const int32_t* inv;   // in-order rank -> heap node
  const double* y;      // n
  const int64_t* yint;  // n, y * 2^sy rounded
  int32_t sy;
  const double* e;      // n x m_e column-major (column 0 = 1)
  const int64_t* eint;  // m_e x n fixed point covariates (column 0 unused)
  const int64_t* gsum;  // p x max(m_e,1) x 2: H and R sums of y (v = 0) and covariate v, fixed point
  const int32_t* se;    // per covariate scale exponent
  const double* ee;     // m_e x m_e upper: E'E (host, FP64)
  const double* ey;     // m_e: E'y
  const double* inv_tau2_e;  // m_e
  double y_absmax;      // max |y|
  const double* e_absmax;    // m_e: max |E column| (1 for the constant)
  double* scratch;      // chains x 2 km: Givens cosines and sines
  double yy;
  // per-chain arrays
  DevModel* cur;        // chains
  DevModel* nm;         // chains
  DevChain* ch;         // chains
  RbParams* rb;         // chains
  double* p_prop;       // chains x p
  double* p_prop_types; // chains x p x n_types
  double* p_rao;        // chains x p
  double* p_rao_types;  // chains x p x n_types
  double* p_r;          // chains x p (last scan; optional output)
  double* p_r_types;    // chains x p x n_types
  double* q_ms;         // chains x 256: q_p_move_size
  double* q_nbs;        // chains x 128
  double* q_nbc;        // chains x 256
  double* r_ms_sum;     // chains x 256
  double* r_ms_n;       // chains x 256
  double* q_p0_ms;      // chains x 256
  int64_t* cadd;        // chains x (p + 1) prefix of dd_add weights (x 2^qs) in in-order
  uint32_t* inbits;     // chains x ceil(p/32): SNP in current model
  uint32_t* basebits;   // chains x ceil(p/32): zeroed in the cadd base
  DevLearned lrn;
  const DevPheno* ph;         // phenotype records
  const uint32_t* pheno_of;   // chains: record of the chain
  double* p_lml;        // chains x p: log posterior odds of inclusion of the last scan, when requested (else null)
  int64_t* tile_sums;   // chains x ceil(p / BMG_REBUILD_TILE): rebuild pass 1
  int32_t* rebuild_active;  // chains: this rebuild covers the chain
  int32_t* model_inds;  // chains x p: current model's index or -1
  int64_t* resid;       // chains x n_pad: fixed-point residual of the last RB step
  double* yhat;         // chains x n: Model::y_hat as compute_pve leaves it
  uint16_t* limbs;      // (chains * L) x n_pad bf16 residual limbs (scan B operand)
  uint32_t n_pad;       // individuals padded to the scan's K multiple
  uint32_t limbs_n;     // L
  uint32_t wait_limit;  // polls of a main-loop mbarrier wait of the tensor-core scan (0: the default)
  // delayed rejection (src/sampler.cpp:882-1049, src/model.hpp:585-844): the
  // exhaustive model of each chain (a copy of the proposed model whose last m
  // terms are permuted to visit all 2^m sub-models) and the sub-models' log
  // probabilities
  uint32_t dr;          // min(delay_rejection, max_move_size); 0: off
  double* dr_l;         // chains x km (km + 1) / 2: packed upper factor
  double* dr_v;         // chains x km
  double* dr_inv;       // chains x km: prior precision per column
  uint8_t* dr_ti;       // chains x km: type index per locus
  uint32_t* dr_x1;      // chains x km: first column of each locus
  uint32_t* dr_x2;      // chains x km: second column (AH)
  double* dr_pm;        // chains x 2^dr
  // missing genotype calls (src/data.cpp:341-376, src/data_model.cpp:30-167,
  // src/sampler.cpp:264-453); miss_total = 0 when the data has none
  uint64_t miss_total;        // G: missing calls in the data
  uint32_t miss_snps;         // SNPs with missing calls
  const int64_t* miss_off;    // p + 1: CSR offsets of each SNP's missing calls
  const uint32_t* miss_ind;   // G: their individuals, ascending per SNP
  const double* miss_prior;   // p x 3: cumulative counts of the calls 0, 1, 2
  const int32_t* miss_rank;   // p: index among the SNPs with missing calls, -1 if none
  const uint32_t* miss_list;  // miss_snps: the SNPs with missing calls, ascending
  uint8_t* miss_val;          // chains x G: imputed genotype (0, 1, 2) of each missing call
  MissCorr* miss_corr;        // chains x miss_snps: corrections of the last RB scan
  long long* miss_fit;        // chains x n_pad: fitted-value corrections of a bulk phase (zero between uses)
  double* miss_yh;            // chains x n: fitted values at missing calls during an imputation step
  long long* miss_inm;        // chains x 2 km: in-model SNPs ascending and their missing calls before them
  DevTrace tr;
};

#endif
