/*
 * bmg.h -- C ABI of libbmg, the GB300 (sm_103a) build of bmagwa's MCMC over
 * SNP inclusion.
 *
 * The reference exposes no library API: its seams are the CLI
 * `bmagwa INIFILE` (src/main.cpp:36-47), the INI schema parsed into
 * bmagwa::Options (src/options.hpp:138-321), the PLINK inputs read by
 * bmagwa::Data (src/data.cpp:141-273), the per-chain
 * bmagwa::Sampler(const Options&, const Data*, const PrecomputedSNPCovariances*)
 * + Sampler::sample() (src/sampler.hpp:107, src/sampler.cpp:551-880), and the
 * binary trace files written by sample() (src/sampler.cpp:547-880).  Each
 * entry point below names the reference interface it replaces.
 *
 * Conventions: plain pointers and sizes, no C++ or torch types.  Host pointers
 * are copied; the caller keeps ownership.  All device memory is owned by the
 * context.  Nothing throws across this boundary: every call returns a
 * bmg_status and bmg_last_error() gives the message.  A context is not
 * thread-safe; use one host thread per context.
 */
#ifndef BMG_H_
#define BMG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bmg_status {
  BMG_OK = 0,
  BMG_EINVAL = 1,       /* bad argument or option (reference: std::runtime_error) */
  BMG_EIO = 2,          /* file missing, truncated, wrong magic */
  BMG_ECUDA = 3,        /* CUDA runtime error or missing device code */
  BMG_ENOTPD = 4,       /* start state not positive definite */
  BMG_ETIMEOUT = 5,     /* a bounded device wait gave up */
  BMG_ENOMEM = 6,
  BMG_EUNSUPPORTED = 7, /* option valid in the reference but not on this path */
  BMG_ENUMERIC = 8      /* NaN met where the reference throws (src/sampler.cpp:213) */
} bmg_status;

/* effect types, numbering of DataModel::ef_t (src/data_model.hpp:41) */
enum { BMG_TYPE_A = 0, BMG_TYPE_H = 1, BMG_TYPE_D = 2, BMG_TYPE_R = 3, BMG_TYPE_AH = 4 };

/* proposal used for additions (BMG_PROPOSAL_ADAPTIVE is the reference's) */
enum { BMG_PROPOSAL_ADAPTIVE = 0, BMG_PROPOSAL_LEARNED = 1 };

/* p-wide scan implementation */
enum { BMG_SCAN_TCGEN05 = 0, BMG_SCAN_SIMT = 1 };

#define BMG_MAX_PATH 1024

/*
 * All INI options of bmagwa::Options (src/options.hpp:41-74), same names and
 * meanings, plus the GPU knobs at the end.  bmg_options_default() fills the
 * reference's defaults; bmg_options_from_ini() parses a reference INI file
 * with the reference's keys, defaults, warnings and validation rules.
 */
typedef struct bmg_options {
  /* [datafiles] */
  char file_fam[BMG_MAX_PATH];
  char file_g[BMG_MAX_PATH];
  char file_e[BMG_MAX_PATH];
  char file_y[BMG_MAX_PATH];
  int32_t recode_g_to_minor_allele_count;
  /* [sizes] */
  uint64_t n;
  uint64_t m_g;
  uint32_t m_e;           /* covariates, excluding the constant */
  /* [model] types, sorted ascending (src/options.hpp:236-252) */
  uint32_t n_types;
  int32_t types[5];
  /* [sampler] */
  int32_t sampler_type;   /* 0 PMV (only PMV is on this path) */
  uint64_t do_n_iter;
  uint64_t n_rao;
  uint64_t n_rao_burnin;
  uint64_t thin;
  uint64_t n_sample_tau2_and_missing;
  uint32_t max_move_size;
  uint32_t max_SNP_neighborhood_size;
  double p_move_size;
  double p_move_size_nbs;
  double p_move_size_nbc;
  int32_t adapt_p_move_size;
  double p_move_size_acpt_goal;
  int32_t adaptation;
  int32_t flat_proposal_dist;
  int32_t save_beta;
  uint64_t verbosity;
  uint32_t delay_rejection;
  /* [thread] */
  char basename[BMG_MAX_PATH];
  uint32_t n_chains;      /* n_threads */
  const uint32_t* seeds;  /* n_chains seeds; caller-owned */
  /* [prior] */
  double e_qg;
  double var_qg;
  double nu_sigma2;
  double s2_sigma2;
  double R2mode_sigma2;
  double mu_alpha;
  double inv_tau2_e_const_val;
  double inv_tau2_e_val;
  int32_t use_individual_tau2;
  double types_prior[5];  /* type_A, type_H, type_D, type_R, type_AH */
  double nu_tau2[4];
  double s2_tau2[4];
  double eh_tau2[4];
  /* GB300 knobs (no reference counterpart) */
  uint32_t max_model_size;  /* columns of X_gamma incl. covariates (ref MAXMODELSIZE 1024) */
  uint32_t scan_limbs;      /* 8-bit residual limbs in the scan GEMM, 3..7 (default 6) */
  int32_t scan_impl;        /* BMG_SCAN_TCGEN05 or BMG_SCAN_SIMT */
  int32_t proposal;         /* BMG_PROPOSAL_ADAPTIVE or BMG_PROPOSAL_LEARNED */
  uint32_t graph_iters;     /* iterations captured per CUDA graph chunk */
  int32_t write_files;      /* 1: bmg_run writes the reference's trace files */
  int32_t quiet;            /* 1: no console warnings */
  /* learned proposal (BMG_PROPOSAL_LEARNED; no reference counterpart) */
  double learned_mix;       /* weight of the MLP part of the add proposal (default 0.3) */
  uint32_t learned_topk;    /* candidate SNPs per chain of the MLP part (default 1024) */
  uint32_t learned_every;   /* RB steps between MLP refreshes during burn-in (default 10) */
  uint32_t learned_steps;   /* optimiser steps per refresh (default 4) */
  double learned_lr;        /* Adam step size (default 1e-3) */
} bmg_options;

/* Trace of a chain over a run chunk, in the reference's file layouts
 * (src/sampler.cpp:686-728; README "Output files and formats"). */
typedef struct bmg_trace_chunk {
  uint32_t chain;
  uint64_t iter0;              /* first iteration of the chunk */
  uint64_t n_iter;             /* per-iteration arrays below have n_iter entries */
  const uint8_t* jumpdistance;
  const uint8_t* move_type;
  const uint8_t* move_size;
  uint64_t n_thin;             /* thinned arrays below have n_thin entries */
  const uint32_t* modelsize;
  uint64_t n_loci;             /* sum of modelsize */
  const uint32_t* loci;
  const uint8_t* types;        /* type index per locus (multi-type runs only) */
  const double* log_likelihood;
  const double* log_prior;
  const double* sigma2;
  const double* alpha;
  const double* pve;           /* 3 per thinned sample */
  uint64_t n_beta;
  const double* beta;          /* save_beta: all coefficients per thinned sample */
} bmg_trace_chunk;

typedef void (*bmg_trace_fn)(void* user, const bmg_trace_chunk* chunk);

typedef struct bmg_trace_sink {
  bmg_trace_fn fn;
  void* user;
} bmg_trace_sink;

typedef struct bmg_ctx bmg_ctx;

/* sizeof(bmg_options) as compiled into the library, for bindings that mirror
 * the struct (no reference counterpart). */
size_t bmg_options_size(void);

/* Reference defaults of every optional key (src/options.hpp:138-321). */
bmg_status bmg_options_default(bmg_options* opt);

/* Parse a reference INI file (replaces bmagwa::Options::Options,
 * src/options.hpp:77-86, parse_options :138-321).  `seeds_buf` receives the
 * seeds (capacity `seeds_cap`); opt->seeds points into it. */
bmg_status bmg_options_from_ini(const char* path, bmg_options* opt,
                                uint32_t* seeds_buf, uint32_t seeds_cap,
                                char* err, size_t err_len);

/* Read the data files an options struct names: .fam phenotypes (and the
 * alternate phenotype file), covariates and the .bed payload, with the
 * reference's matching and error rules (replaces Data::read_fam/read_y/
 * read_e/read_g, src/data.cpp:141-273).  packed: m_g*ceil(n/4) bytes;
 * y: n doubles; e: n*m_e doubles column-major (NULL when m_e == 0). */
bmg_status bmg_read_plink(const bmg_options* opt, uint8_t* packed, double* y, double* e,
                          char* err, size_t err_len);

/* Create a context on the current CUDA device (replaces the per-chain
 * Sampler construction, src/sampler.hpp:107-282, for all chains at once). */
bmg_status bmg_create(const bmg_options* opt, bmg_ctx** out);

/* Copy SNP-major packed PLINK genotypes (the .bed payload after its 3 magic
 * bytes: p rows of ceil(n/4) bytes) to the device (replaces Data::read_g,
 * src/data.cpp:245-273, and the recode/missing passes :324-376). */
bmg_status bmg_load_bed(bmg_ctx* ctx, const uint8_t* packed, uint64_t n, uint64_t p);

/* Phenotypes: n_pheno rows of n doubles (replaces Data::read_fam/read_y,
 * src/data.cpp:141-200).  Chain c uses phenotype c % n_pheno.  `mask` is
 * optional: n_pheno rows of n bytes, 1 = individual kept for that phenotype
 * (no reference counterpart; the reference needs one run per phenotype). */
bmg_status bmg_set_phenotypes(bmg_ctx* ctx, const double* y, const uint8_t* mask,
                              uint32_t n_pheno);

/* Covariates without the constant column: m_e columns of n doubles,
 * column-major (replaces Data::read_e, src/data.cpp:202-243). */
bmg_status bmg_set_covariates(bmg_ctx* ctx, const double* e, uint32_t m_e);

/* Per-SNP sums and centred second moments of every allowed term
 * (replaces PrecomputedSNPCovariances::precompute,
 * src/precomputed_snp_covariances.hpp:95-131) and the start state of every
 * chain (Sampler ctor + initialize_p_proposal_flat, src/sampler.hpp:351-362). */
bmg_status bmg_precompute(bmg_ctx* ctx);

/* Read back the precomputed per-SNP values: m_g rows of `offset` doubles in
 * the reference's layout (PrecomputedSNPCovariances::xx, :42-84). */
bmg_status bmg_get_precomputed(bmg_ctx* ctx, double* xx, uint32_t* offset);

/* Rao-Blackwellised single-SNP scan of every chain at its current state
 * (replaces RaoBlackwellizer::p_raoblackwell, src/sampler.cpp:32-261).
 * p_r: n_chains x m_g; p_r_types: n_chains x m_g x n_types (may be NULL). */
bmg_status bmg_scan(bmg_ctx* ctx, double* p_r, double* p_r_types);

/* The same scan with the per-SNP log posterior odds of inclusion written to
 * logodds (chains x m_g, chain-major): log of p_r / (1 - p_r), computed
 * before the logistic, the per-SNP Bayes factor with its prior odds
 * (src/sampler.cpp:193-195; with several effect types log sum_t exp,
 * :241-255).  No
 * counterpart entry point in the reference; its error against the FP64
 * oracle is the one the parity tests bound. */
bmg_status bmg_scan_logodds(bmg_ctx* ctx, double* logodds);

/* The Rao-Blackwellised scan of every chain against fitted values the caller
 * gives instead of the model's (no counterpart entry point in the reference:
 * RaoBlackwellizer::p_raoblackwell, src/sampler.cpp:32-261, called with this
 * y_hat and sigma2; a parity aid).  y_hat: n doubles, the same for every
 * chain.  Every chain's current sigma2 is set to sigma2 (> 0) and stays so.
 * p_r and logodds (either may be NULL) receive chains x m_g values as
 * bmg_scan and bmg_scan_logodds write them. */
bmg_status bmg_scan_yhat(bmg_ctx* ctx, const double* y_hat, double sigma2, double* p_r, double* logodds);

/* The exact change of every chain's log marginal likelihood from adding each
 * single term of each SNP outside its model (no counterpart entry point in
 * the reference: Model::update_likelihood_on_add, src/model.hpp:432-506,
 * evaluated for every candidate without changing the model).  dlml receives
 * chains x m_g x terms doubles (terms: the allowed single codings A, H, D, R
 * in that order; AH contributes A and H), NaN for SNPs in the model and -inf
 * where the enlarged system is not positive definite.  The prior precision
 * of a term is the chain's shared tau2 value.  Models of more than 128
 * columns return BMG_EUNSUPPORTED. */
bmg_status bmg_scan_schur(bmg_ctx* ctx, double* dlml);

/* Learned proposal (BMG_PROPOSAL_LEARNED; no reference counterpart).
 * Snapshot: the MLP's MLP_NPAR = 18817 FP32 parameters (W1 128x16, b1 128,
 * W2 128x128, b2 128, w3 128, b3), its logits at the current state
 * (chains x m_g), the features of the current state (chains x m_g x 16), and
 * the candidate tables (chains x topk SNPs and weights, chains counts); any
 * pointer may be NULL. */
bmg_status bmg_learned_snapshot(bmg_ctx* ctx, float* theta, float* logit, float* features, uint32_t* t_snp,
                                double* t_s, uint32_t* t_n);

/* The gradient of the training loss (mean binary cross-entropy of the MLP's
 * output against the chain's p_proposal) over an explicit list of rows
 * (n_rows pairs chain, SNP) at the current parameters, written to grad
 * (18817 floats); the parameters do not change. */
bmg_status bmg_learned_grad(bmg_ctx* ctx, const uint32_t* rows, uint32_t n_rows, float* grad);

/* Advance every chain by n_iter MCMC iterations (replaces the main loop of
 * Sampler::sample, src/sampler.cpp:626-834).  Traces go to `sink` (may be
 * NULL) and, with opt.write_files, to the reference's files. */
bmg_status bmg_run(bmg_ctx* ctx, uint64_t n_iter, const bmg_trace_sink* sink);

/* Current state of one chain (the fields of bmagwa::Model the traces show). */
typedef struct bmg_chain_state {
  uint32_t model_size;
  double log_likelihood;
  double log_prior;
  double sigma2;
  double alpha;
  uint64_t n_iter;
  uint64_t n_accepted;
  double p_move_size;
  uint64_t rng_draws;     /* logical random draws so far (the stream position) */
} bmg_chain_state;

/* loci (capacity loci_cap) receives the model's SNPs in model order. */
bmg_status bmg_get_state(bmg_ctx* ctx, uint32_t chain, bmg_chain_state* st,
                         uint32_t* loci, uint8_t* type_inds, uint32_t loci_cap);

/* Rao-Blackwellised posterior of a chain (the _rao.dat / _rao_types.dat
 * payloads, src/sampler.cpp:846-858).  p_rao_types may be NULL. */
bmg_status bmg_get_rao(bmg_ctx* ctx, uint32_t chain, double* p_rao, double* p_rao_types);

/* The same for every chain in one call: p_rao receives chains x m_g values
 * (chain-major), p_rao_types chains x m_g x n_types or is NULL.  The copy is
 * pipelined through the pinned staging buffers (no counterpart in the
 * reference, which writes one _rao.dat per chain). */
bmg_status bmg_get_rao_all(bmg_ctx* ctx, double* p_rao, double* p_rao_types);

/* Adaptive proposal of a chain: the running mean p_proposal of the
 * Rao-Blackwellised probabilities that sets the add/remove weights
 * (Sampler::save_p_proposal, src/sampler.hpp:363-383).  p_prop_types may be NULL. */
bmg_status bmg_get_proposal(bmg_ctx* ctx, uint32_t chain, double* p_prop, double* p_prop_types);

/* Rao-Blackwellised probabilities of the last scan inside bmg_run (the
 * p_r_ the reference averages, src/sampler.cpp:731-757).  p_r_types may be NULL. */
bmg_status bmg_get_last_scan(bmg_ctx* ctx, uint32_t chain, double* p_r, double* p_r_types);

/* Write a chain's _rao.dat, _rao_types.dat, _samplerstats.txt and _prior.txt
 * under opt.basename (src/sampler.cpp:838-858, src/sampler.hpp:384-390). */
bmg_status bmg_finish(bmg_ctx* ctx);

/* Device time of the phases of bmg_run since the last bmg_reset_timings, in
 * milliseconds: [0] move kernel, [1] scan, [2] proposal rebuild, [3] total. */
bmg_status bmg_get_timings(bmg_ctx* ctx, double* ms4);

/* var_x, mean_x, var_y, y'y of the loaded data (src/data.hpp:66-71; the
 * reference prints the first three at start, src/main.cpp:58-62). */
bmg_status bmg_get_data_stats(bmg_ctx* ctx, double* out4);

/* Zero the phase timers; n_scans (may be NULL) receives the scans since the
 * last reset. */
bmg_status bmg_reset_timings(bmg_ctx* ctx, uint64_t* n_scans);

/* Kernels of this library launched by ctx since the last bmg_reset_timings
 * (no counterpart in the reference; a measurement aid). */
bmg_status bmg_get_launch_count(bmg_ctx* ctx, uint64_t* n_launches);

/* Self-test of the scan's table-driven exp (no counterpart in the reference):
 * out[i] = exp(a[i]) as the posterior epilogue evaluates it, for host arrays
 * of n arguments with |a[i]| <= 700 (others give BMG_EINVAL).  Uses the
 * current CUDA device and allocates 16 n bytes there for the call. */
bmg_status bmg_selftest_exp(const double* a, double* out, size_t n);

/* Launch shape of the tensor-core scan (no counterpart in the reference).
 * The first scans of a context time each shape once and keep the fastest;
 * every shape gives the same results bit for bit.  variant is -1 while
 * tuning; BMG_SCAN_VARIANT=<i> in the environment at bmg_create fixes it. */
bmg_status bmg_get_scan_shape(bmg_ctx* ctx, int32_t* variant, char* name, size_t name_len);

/* The tuner's time of each launch shape (no counterpart in the reference):
 * ms[i] = the fastest of its tuning scans in milliseconds, -1 if not timed
 * (yet).  Writes min(n, shapes) entries; *n_shapes (may be NULL) receives
 * the number of shapes. */
bmg_status bmg_get_scan_tuning(bmg_ctx* ctx, float* ms, int32_t n, int32_t* n_shapes);

/* Description of launch shape `shape` (0 .. n_shapes - 1). */
bmg_status bmg_get_scan_shape_name(int32_t shape, char* name, size_t name_len);

/* Per-SNP precomputed sums, allocating nothing (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc, e.g. code running in
 * another framework's memory pool or while a stream is being captured.
 * Inputs and outputs are the caller's device buffers: d_packed holds p rows of
 * ceil(n/4) bytes (the .bed payload), d_out receives p x offset doubles in the
 * layout bmg_get_precomputed() returns (offset is written to *offset_out),
 * d_flag one int32 set to 1 if any genotype call is missing (missing calls
 * count as 0, as in the reference's precomputation).  `stream` is a
 * cudaStream_t or NULL.  Working memory is a fixed array inside the library
 * of 3 x 2^20 int32 (12 MB per device, kept until the process exits); p above
 * 2^20, or n above 2^31 - 1, returns BMG_EINVAL.  The first call on each
 * device looks up that array's device address, so make the first call before
 * capturing a stream.  Calls that overlap on the GPU share the array and
 * race; calls ordered on one stream do not.  A failed call leaves its message
 * for bmg_last_error(NULL) on the calling thread. */
bmg_status bmg_precompute_noalloc(const uint8_t* d_packed, uint64_t n, uint64_t p, int32_t recode,
                                  const int32_t* types, uint32_t n_types, double* d_out,
                                  uint32_t* offset_out, int32_t* d_flag, void* stream);

/* Message of the last failed call on ctx; with ctx NULL, the message of the
 * last failed call on the calling thread that has no context (bmg_create,
 * bmg_precompute_noalloc). */
const char* bmg_last_error(const bmg_ctx* ctx);
const char* bmg_status_string(bmg_status s);
void bmg_destroy(bmg_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* BMG_H_ */
