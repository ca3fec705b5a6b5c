// libbmg host side: context, device memory, the iteration schedule and the
// reference's output files.
//
// Launch schedule per chunk of iterations: the move kernel (one CTA per
// chain) runs iterations up to and including the next Rao-Blackwellisation
// step (src/sampler.cpp:731: (iter + 1) % n_rao == 0); then the p-wide scan
// and the proposal-prefix rebuild run for all chains at once.  The schedule
// is the same for every chain, so it is known on the host; the launches of a
// chunk are captured once in a CUDA graph and replayed.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <memory>
#include <sstream>
#include <thread>
#include <string>
#include <cstdlib>
#include <vector>

#include <cuda_runtime.h>

#include "bmg.h"
#include "bmg_internal.h"
#include "dev/state.h"

extern "C" __global__ void bmg_prep_kernel(uint8_t* geno, uint64_t n, uint64_t p, uint32_t gs,
                                           int recode, int32_t* cnt, int32_t* missing);
extern "C" __global__ void bmg_trace_reset_kernel(DevChain* ch, int n_chains);
extern "C" __global__ void bmg_mask_counts_kernel(const uint8_t* geno, uint32_t gs, uint64_t p, const uint64_t* mask2,
                                                  uint32_t n_samples, int32_t* cnt);
extern "C" __global__ void bmg_tail_kernel(uint8_t* g, uint64_t p, uint64_t gs, uint64_t last, uint8_t keep);
extern "C" __global__ void bmg_pre_df_kernel(const double* pre, uint64_t p, uint32_t offset, uint32_t off,
                                             float4* out);
extern "C" __global__ void bmg_pre_kernel(const int32_t* cnt, uint64_t p, uint32_t n_samples, const double* n_of,
                                          int allow_mask, int ah, int offset, double* pre);
extern "C" __global__ void bmg_gsum_kernel(const uint8_t* geno, uint64_t n, uint64_t p, uint32_t gs,
                                           const int64_t* yint, const int64_t* eint, uint32_t nv, int64_t* gsum);
extern "C" __global__ void bmg_init_kernel(DevConst K);
extern "C" __global__ void bmg_rbprep_kernel(DevConst K, int from_yhat, double yhat_absmax);
extern "C" __global__ void bmg_set_sigma2_kernel(DevConst K, double sigma2);
extern "C" __global__ void bmg_miss_scan_kernel(DevConst K);
extern "C" __global__ void bmg_move_kernel(DevConst K, int max_iters);
extern "C" __global__ void bmg_scan_simt_kernel(DevConst K, const int64_t* resid_t);
extern "C" __global__ void bmg_resid_transpose_kernel(DevConst K, int64_t* resid_t);
extern "C" __global__ void bmg_rebuild_sums_kernel(DevConst K, int force);
extern "C" __global__ void bmg_rebuild_write_kernel(DevConst K);
extern "C" cudaError_t bmg_move_configure(size_t* smem_bytes);
// tensor-core scan (scan_tc.cu)
extern "C" int bmg_scan_tc_launch(const DevConst* K, cudaStream_t stream, int variant);
extern "C" int bmg_scan_tc_variants();
extern "C" cudaError_t bmg_mlp_init(const DevConst* K, int32_t* adam_t, cudaStream_t s);
extern "C" cudaError_t bmg_mlp_refresh(const DevConst* K, uint32_t km, int steps, float lr, int32_t* adam_t,
                                       cudaStream_t s);
extern "C" cudaError_t bmg_mlp_features(const DevConst* K, float* out, cudaStream_t s);
extern "C" cudaError_t bmg_mlp_forward(const DevConst* K, cudaStream_t s);
extern "C" cudaError_t bmg_mlp_grad(const DevConst* K, const int32_t* adam_t, const uint32_t* rows, uint32_t n,
                                    cudaStream_t s);
extern "C" int bmg_schur_launch(const DevConst* K, const int* xcols, uint16_t** bm, size_t* bm_cap, double* out,
                                cudaStream_t stream);
extern "C" void bmg_scan_tc_variant_name(int v, char* buf, size_t len);
extern "C" int bmg_scan_tc_variant_redundant(const DevConst* K, int v);
extern "C" int bmg_scan_tc_supported(const DevConst* K);

using bmg_host::bmg_error;

namespace {

#define CK(x)                                                                       \
  do {                                                                              \
    cudaError_t e_ = (x);                                                           \
    if (e_ != cudaSuccess)                                                          \
      throw bmg_error(BMG_ECUDA, std::string(#x) + ": " + cudaGetErrorString(e_));  \
  } while (0)

// after a kernel launch: the launch error, and with sync_check the kernel's
// own execution error, named
#define LAUNCHED(ctx, name)                                                                      \
  do {                                                                                           \
    cudaError_t e_ = cudaGetLastError();                                                         \
    if ((ctx)->capturing) ++(ctx)->graph_launches; else ++(ctx)->n_launches;                     \
    if (e_ == cudaSuccess && (ctx)->sync_check) e_ = cudaStreamSynchronize((ctx)->stream);       \
    if (e_ != cudaSuccess) throw bmg_error(BMG_ECUDA, std::string(name) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct ChainFiles {
  std::ofstream log, loci, modelsize, jumpdistance, log_likelihood, log_prior, move_type,
      move_size, pve, alpha, sigma2, types, beta;
  bool open = false;
};

const char* kTypeName[5] = {"A", "H", "D", "R", "AH"};

}  // namespace

// One chunk of iterations as a list of segments: seg iterations of the move
// kernel, then (rb) the scan and the prefix rebuild.
struct Segment {
  uint64_t iters;
  bool rb;
  bool refresh;  // learned proposal refreshed after the RB step
  bool operator==(const Segment& o) const { return iters == o.iters && rb == o.rb && refresh == o.refresh; }
};

struct bmg_ctx {
  bmg_options opt;
  std::vector<uint32_t> seeds;
  std::string err;
  uint64_t n = 0, p = 0;
  uint32_t C = 0, km = 0, L = 6, gs = 0, n_pad = 0;
  bool have_geno = false, have_y = false, have_e = false, ready = false;
  std::vector<int32_t> cnt_h;
  std::vector<double> y_h, e_h, pre_h;
  double var_x = 0, mean_x = 0, var_y = 0, yy = 0;
  // several phenotypes (one chain each): per sample the individuals, values
  // (zero outside), and sums; record k of K.ph is built from these
  bool multi = false;
  std::vector<uint8_t> ph_mask;        // n_pheno x n: 1 = in the sample
  std::vector<double> ph_n, ph_yy, ph_var_y, ph_amax, ph_ysum;
  std::vector<int32_t> ph_sy;
  double* ph_y_dev = nullptr;          // n_pheno x n
  int64_t* ph_yint_dev = nullptr;      // n_pheno x n
  double g_a = 0, g_b = 0, s2_sigma2 = 0, s2_tau2[4] = {0, 0, 0, 0};
  std::vector<void*> allocs;
  DevConst K;
  int64_t* resid_t = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<ChainFiles> files;
  std::vector<DevChain> ch_h;
  double ms[4] = {0, 0, 0, 0};
  uint64_t n_scans = 0;
  size_t move_smem = 0;   // dynamic shared memory of a move CTA
  bool sync_check = false; // BMG_SYNC_CHECK=1: synchronise after every launch
  uint64_t n_launches = 0; // kernels of this library launched since the last counter reset
  // launch-shape autotuner of the tensor-core scan: the first scan warms
  // up, the next ones time one shape each, then the fastest is kept
  bool eager = false;      // BMG_EAGER=1: no CUDA graphs
  bool capturing = false;  // a chunk is being captured into a graph
  std::vector<cudaEvent_t> seg_ev;             // 4 events per segment of a chunk
  cudaGraphExec_t graph_exec = nullptr;        // the captured chunk
  std::vector<Segment> graph_segs;             // ... and its segment pattern
  uint64_t graph_launches = 0;                 // kernels in the captured chunk
  double* lml_buf = nullptr;                   // per-SNP log odds of the scans (bmg_scan_logodds, learned proposal)
  double* yhat_given = nullptr;                // chains x n fitted values of bmg_scan_yhat
  std::vector<int64_t> miss_off;               // missing calls per SNP (CSR offsets, p + 1)
  std::vector<uint32_t> miss_ind;              // their individuals
  std::vector<double> miss_prior;              // p x 3 cumulative counts of the calls 0, 1, 2
  uint32_t wait_limit = 0;                     // main-loop wait bound of the tensor-core scan (0: default)
  uint32_t dr = 0;                             // delayed rejection: largest move enumerated (0: off)
  int32_t* adam_t = nullptr;                   // learned proposal: optimiser step counter (device)
  uint64_t rb_steps = 0;                       // RB steps issued by bmg_run
  double* schur_out = nullptr;                 // bmg_scan_schur output on the device
  uint16_t* schur_bm = nullptr;                // its B operand (model columns), grown on demand
  size_t schur_bm_cap = 0;
  int tc_forced = -1;      // BMG_SCAN_VARIANT
  int tc_variant = -1;     // chosen shape (-1 while tuning)
  int tc_tuned = 0;        // tuning scans issued
  int tc_pending = -1;     // shape whose timing events are not read yet
  cudaEvent_t tc_ev[2] = {nullptr, nullptr};
  std::vector<float> tc_ms;
  std::vector<int> tc_cands;  // shapes the tuner times
  cudaEvent_t ev[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  uint64_t n_iter = 0;
  time_t t_start = 0;
  int max_ms = 0;
  // host copies of the trace buffers
  std::vector<uint8_t> h_jump, h_mtype, h_msize, h_types;
  std::vector<uint32_t> h_msz, h_loci;
  std::vector<double> h_ll, h_lp, h_s2, h_alpha, h_pve, h_beta, h_log;

  template <class T>
  T* dalloc(size_t count, bool zero = true)
  {
    void* ptr = nullptr;
    size_t bytes = std::max<size_t>(1, count * sizeof(T));
    CK(cudaMalloc(&ptr, bytes));
    allocs.push_back(ptr);
    // on the context's own (non-blocking) stream: a legacy-stream memset is
    // not ordered with the uploads that follow on `stream`
    if (zero) CK(cudaMemsetAsync(ptr, 0, bytes, stream));
    return static_cast<T*>(ptr);
  }
  // pinned host staging for uploads and read-backs: two buffers (chunks of
  // an upload alternate between them while the other's DMA runs)
  uint8_t* stage[2] = {nullptr, nullptr};
  size_t stage_cap = 0;
  cudaEvent_t stage_ev[2] = {nullptr, nullptr};
  void ensure_stage(size_t bytes)
  {
    if (stage_cap >= bytes) return;
    for (int b = 0; b < 2; ++b) {
      if (stage[b]) {
        CK(cudaEventSynchronize(stage_ev[b]));
        cudaFreeHost(stage[b]);
        stage[b] = nullptr;
      }
    }
    stage_cap = 0;
    for (int b = 0; b < 2; ++b) {
      CK(cudaMallocHost(reinterpret_cast<void**>(&stage[b]), bytes));
      if (!stage_ev[b]) CK(cudaEventCreateWithFlags(&stage_ev[b], cudaEventDisableTiming));
      CK(cudaEventRecord(stage_ev[b], stream));
    }
    stage_cap = bytes;
  }
  ~bmg_ctx()
  {
    for (int b = 0; b < 2; ++b) {
      if (stage_ev[b]) cudaEventSynchronize(stage_ev[b]);
      if (stage[b]) cudaFreeHost(stage[b]);
      if (stage_ev[b]) cudaEventDestroy(stage_ev[b]);
    }
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : tc_ev)
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : seg_ev) cudaEventDestroy(e);
    if (schur_bm) cudaFree(schur_bm);
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    for (void* a : allocs) cudaFree(a);
    if (stream) cudaStreamDestroy(stream);
  }
};

static bmg_status fail(bmg_ctx* ctx, const bmg_error& e)
{
  if (ctx) ctx->err = e.what();
  return e.status;
}

#define API_BEGIN try {
#define API_END                                                    \
  }                                                                \
  catch (const bmg_error& e) { return fail(ctx, e); }             \
  catch (const std::exception& e) { return fail(ctx, bmg_error(BMG_EINVAL, e.what())); }

// ------------------------------------------------------------------ helpers

/* src/utils.cpp:144-152 */
static void geometric_cdf(int maxsize, double p, double* values)
{
  double q = 1 - p, qp = q;
  for (int i = 0; i < maxsize; ++i) {
    values[i] = 1 - q;
    q *= qp;
  }
}

// in-order rank of every node of a heap-shaped binary tree with p nodes
static void inorder_ranks(uint64_t p, std::vector<int32_t>& pos, std::vector<int32_t>& inv)
{
  pos.assign(p, 0);
  inv.assign(p, 0);
  std::vector<uint64_t> stack;
  uint64_t node = 0;
  int32_t rank = 0;
  while (node < p || !stack.empty()) {
    while (node < p) {
      stack.push_back(node);
      node = 2 * node + 1;
    }
    node = stack.back();
    stack.pop_back();
    pos[node] = rank;
    inv[rank] = (int32_t)node;
    ++rank;
    node = 2 * node + 2;
  }
}

static int fixed_exponent(double absmax, uint64_t n)
{
  // largest s with n * absmax * 2^s < 2^61 (so sums of 2|x| fit in int64)
  if (!(absmax > 0)) return 0;
  return (int)std::floor(61.0 - std::log2((double)n) - std::log2(absmax)) - 1;
}

static void check_ready(bmg_ctx* ctx)
{
  if (!ctx->ready) throw bmg_error(BMG_EINVAL, "bmg_precompute has not run");
}

static void device_error_check(bmg_ctx* ctx)
{
  CK(cudaMemcpyAsync(ctx->ch_h.data(), ctx->K.ch, sizeof(DevChain) * ctx->C, cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (uint32_t c = 0; c < ctx->C; ++c) {
    int e = ctx->ch_h[c].error;
    if (e == BMG_DERR_NONE) continue;
    const char* what = "device error";
    bmg_status st = BMG_ECUDA;
    switch (e) {
      case BMG_DERR_CAPACITY: what = "Not enough memory for adding term (max_model_size)"; st = BMG_EINVAL; break;
      case BMG_DERR_NAN: what = "raob max_types is nan"; st = BMG_ENUMERIC; break;
      case BMG_DERR_RNG: what = "gamma sampler ran out of attempts"; st = BMG_ENUMERIC; break;
      case BMG_DERR_PEND: what = "proposal flip list overflow"; st = BMG_ECUDA; break;
      case BMG_DERR_TRACE: what = "trace buffer overflow"; st = BMG_ECUDA; break;
      case BMG_DERR_REMSET: what = "model too large for the removal proposal set"; st = BMG_EINVAL; break;
      case BMG_DERR_START: what = "Sampler cannot start from non-finite likelihood."; st = BMG_ENOTPD; break;
      case BMG_DERR_TIMEOUT: what = "a bounded device wait gave up"; st = BMG_ETIMEOUT; break;
    }
    throw bmg_error(st, std::string(what) + " (chain " + std::to_string(c) + ")");
  }
}

// ---------------------------------------------------------------- create

// message of the last failed call without a context on this thread
static thread_local std::string g_create_error;

void bmg_host::set_thread_error(const std::string& msg) { g_create_error = msg; }

extern "C" bmg_status bmg_create(const bmg_options* opt, bmg_ctx** out)
{
  bmg_ctx* ctx = nullptr;
  try {
    if (!opt || !out) throw bmg_error(BMG_EINVAL, "null argument");
    std::unique_ptr<bmg_ctx> c(new bmg_ctx());
    ctx = c.get();
    c->opt = *opt;
    if (opt->n_chains == 0 || !opt->seeds) throw bmg_error(BMG_EINVAL, "n_chains and seeds are required");
    c->seeds.assign(opt->seeds, opt->seeds + opt->n_chains);
    c->opt.seeds = c->seeds.data();
    if (opt->sampler_type != 0)
      throw bmg_error(BMG_EUNSUPPORTED, "only the PMV sampler runs on the GPU path");
    if (opt->proposal != BMG_PROPOSAL_ADAPTIVE && opt->proposal != BMG_PROPOSAL_LEARNED)
      throw bmg_error(BMG_EINVAL, "proposal must be BMG_PROPOSAL_ADAPTIVE or BMG_PROPOSAL_LEARNED");
    if (opt->proposal == BMG_PROPOSAL_LEARNED &&
        (!(opt->learned_mix >= 0 && opt->learned_mix < 1) || opt->learned_topk == 0 || opt->learned_topk > 65536 ||
         opt->learned_every == 0 || !(opt->learned_lr > 0)))
      throw bmg_error(BMG_EINVAL, "learned proposal: mix in [0, 1), topk in 1..65536, every >= 1, lr > 0");
    if (opt->n == 0 || opt->m_g == 0) throw bmg_error(BMG_EINVAL, "n and m_g must be positive");
    if (opt->n_types == 0 || opt->n_types > 5) throw bmg_error(BMG_EINVAL, "types");
    if (opt->thin == 0 || opt->n_rao == 0 || opt->n_sample_tau2_and_missing == 0)
      throw bmg_error(BMG_EINVAL, "thin, n_rao and n_sample_tau2_and_missing must be positive");
    if (opt->n_rao % opt->thin != 0) throw bmg_error(BMG_EINVAL, "Config error: n_rao should be a multiple of thin");
    // the state-change move permutes 2 x neighbourhood positions in a
    // fixed-size on-chip list
    if (2ull * opt->max_SNP_neighborhood_size > BMG_MAX_MS + 1)
      throw bmg_error(BMG_EINVAL, "max_SNP_neighborhood_size above " + std::to_string((BMG_MAX_MS + 1) / 2) +
                                      " is not supported");
    c->n = opt->n;
    c->p = opt->m_g;
    c->C = opt->n_chains;
    c->km = opt->max_model_size ? opt->max_model_size : 1024;
    c->L = opt->scan_limbs ? opt->scan_limbs : 6;
    if (c->L < 3 || c->L > 7) throw bmg_error(BMG_EINVAL, "scan_limbs must be 3..7");
    c->max_ms = (int)std::min<uint64_t>(std::min<uint64_t>(c->p, 255), opt->max_move_size);
    // delayed rejection enumerates 2^m sub-models of a rejected move of m
    // SNPs (src/sampler.hpp:163-169: m <= min(delay_rejection, max_move_size))
    c->dr = (uint32_t)std::min<uint64_t>((uint64_t)c->max_ms, opt->delay_rejection);
    if (c->dr > BMG_DR_MAX)
      throw bmg_error(BMG_EUNSUPPORTED, "delayed rejection above " + std::to_string(BMG_DR_MAX) +
                                            " SNPs per move is not on the GPU path");
    if (c->km + (uint32_t)c->max_ms > BMG_REMSET_MAX)
      throw bmg_error(BMG_EINVAL, "max_model_size + max_move_size exceeds the device limit");
    if (c->km < opt->m_e + 3) throw bmg_error(BMG_EINVAL, "max_model_size too small");
    if (c->p >= (1ull << 31)) throw bmg_error(BMG_EINVAL, "m_g too large");
    c->n_pad = (uint32_t)(((c->n + 127) / 128) * 128);
    c->gs = c->n_pad / 4;
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    const char* sc = std::getenv("BMG_SYNC_CHECK");
    c->sync_check = sc && sc[0] && sc[0] != '0';
    const char* eg = std::getenv("BMG_EAGER");
    c->eager = eg && eg[0] && eg[0] != '0';
    // BMG_WAIT_LIMIT=<polls>: a shorter bound on the tensor-core scan's
    // main-loop waits (a test makes them run out and checks BMG_ETIMEOUT)
    const char* wl = std::getenv("BMG_WAIT_LIMIT");
    if (wl && wl[0]) c->wait_limit = (uint32_t)std::max(1L, std::atol(wl));
    const char* sv = std::getenv("BMG_SCAN_VARIANT");
    if (sv && sv[0]) c->tc_forced = std::max(0, std::min(bmg_scan_tc_variants() - 1, std::atoi(sv)));
    c->ch_h.resize(c->C);
    *out = c.release();
    return BMG_OK;
  } catch (const bmg_error& e) {
    if (out) *out = nullptr;
    g_create_error = e.what();
    return e.status;
  } catch (const std::exception& e) {
    if (out) *out = nullptr;
    g_create_error = e.what();
    return BMG_EINVAL;
  }
}

extern "C" void bmg_destroy(bmg_ctx* ctx) { delete ctx; }

extern "C" const char* bmg_last_error(const bmg_ctx* ctx)
{
  return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

extern "C" const char* bmg_status_string(bmg_status s)
{
  switch (s) {
    case BMG_OK: return "BMG_OK";
    case BMG_EINVAL: return "BMG_EINVAL";
    case BMG_EIO: return "BMG_EIO";
    case BMG_ECUDA: return "BMG_ECUDA";
    case BMG_ENOTPD: return "BMG_ENOTPD";
    case BMG_ETIMEOUT: return "BMG_ETIMEOUT";
    case BMG_ENOMEM: return "BMG_ENOMEM";
    case BMG_EUNSUPPORTED: return "BMG_EUNSUPPORTED";
    case BMG_ENUMERIC: return "BMG_ENUMERIC";
  }
  return "unknown";
}

// ------------------------------------------------------------------ data

extern "C" bmg_status bmg_load_bed(bmg_ctx* ctx, const uint8_t* packed, uint64_t n, uint64_t p)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  if (!packed) throw bmg_error(BMG_EINVAL, "null genotypes");
  if (n != ctx->n || p != ctx->p) throw bmg_error(BMG_EINVAL, "genotype sizes differ from the options");
  const uint64_t stride = (n + 3) / 4, gs = ctx->gs;
  const int tail = (int)(n % 4);
  // rows of `stride` bytes into the zeroed, padded device layout by pitched
  // copies from pinned staging chunks (host copies by several threads, the
  // DMA of one chunk overlapping the host copy of the next); the unused
  // codes of a row's last byte are then cleared
  uint8_t* g = ctx->dalloc<uint8_t>(gs * p);
  int32_t* cnt = ctx->dalloc<int32_t>(2 * p);
  int32_t* miss = ctx->dalloc<int32_t>(p);
  {
    const size_t chunk_rows = std::min<size_t>(p, std::max<size_t>(1, (size_t(32) << 20) / stride));
    ctx->ensure_stage(chunk_rows * stride);
    const unsigned nth = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
    int b = 0;
    for (uint64_t j0 = 0; j0 < p; j0 += chunk_rows, b ^= 1) {
      const size_t rows = std::min<uint64_t>(chunk_rows, p - j0), bytes = rows * stride;
      CK(cudaEventSynchronize(ctx->stage_ev[b]));
      uint8_t* dst = ctx->stage[b];
      const uint8_t* src = packed + j0 * stride;
      std::vector<std::thread> th;
      const size_t part = (bytes + nth - 1) / nth;
      for (unsigned t = 0; t < nth && t * part < bytes; ++t)
        th.emplace_back([=] { std::memcpy(dst + t * part, src + t * part, std::min(part, bytes - t * part)); });
      for (auto& x : th) x.join();
      CK(cudaMemcpy2DAsync(g + j0 * gs, gs, dst, stride, stride, rows, cudaMemcpyHostToDevice, ctx->stream));
      CK(cudaEventRecord(ctx->stage_ev[b], ctx->stream));
    }
  }
  if (tail) {
    bmg_tail_kernel<<<(unsigned)std::min<uint64_t>((p + 255) / 256, 152 * 16), 256, 0, ctx->stream>>>(
        g, p, gs, stride - 1, (uint8_t)((1u << (2 * tail)) - 1));
    LAUNCHED(ctx, "bmg_tail_kernel");
  }
  unsigned blocks = (unsigned)std::min<uint64_t>((p + 7) / 8, 152 * 16);
  bmg_prep_kernel<<<blocks, 256, 0, ctx->stream>>>(g, n, p, ctx->gs, ctx->opt.recode_g_to_minor_allele_count,
                                                   cnt, miss);
  LAUNCHED(ctx, "bmg_prep_kernel");
  ctx->cnt_h.resize(2 * p);
  std::vector<int32_t> miss_h(p);
  CK(cudaMemcpyAsync(ctx->cnt_h.data(), cnt, 8 * p, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(miss_h.data(), miss, 4 * p, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  // missing calls (src/data.cpp:341-376): per SNP the individuals without a
  // call, ascending (CSR), and the cumulative counts of the calls 0, 1, 2
  // after the recode, the prior of their imputation
  ctx->miss_off.assign(p + 1, 0);
  for (uint64_t j = 0; j < p; ++j) ctx->miss_off[j + 1] = ctx->miss_off[j] + miss_h[j];
  const uint64_t G = (uint64_t)ctx->miss_off[p];
  ctx->miss_ind.clear();
  ctx->miss_prior.clear();
  if (G) {
    ctx->miss_ind.resize(G);
    ctx->miss_prior.assign(3 * p, 0.0);
    for (uint64_t j = 0; j < p; ++j) {
      const double n1 = ctx->cnt_h[2 * j], n2 = ctx->cnt_h[2 * j + 1];
      const double n0 = (double)n - miss_h[j] - n1 - n2;
      ctx->miss_prior[3 * j] = n0;
      ctx->miss_prior[3 * j + 1] = n0 + n1;
      ctx->miss_prior[3 * j + 2] = n0 + n1 + n2;
      if (!miss_h[j]) continue;
      const uint8_t* row = packed + j * stride;
      int64_t q = ctx->miss_off[j];
      for (uint64_t i = 0; i < n; ++i)
        if (((row[i >> 2] >> (2 * (i & 3))) & 3) == 1) ctx->miss_ind[q++] = (uint32_t)i;
    }
  }
  /* src/data.cpp:403-434 from the counts over each SNP's calls */
  double total_var = 0, total_mean = 0;
  uint64_t nv = 0, nm = 0;
  for (uint64_t j = 0; j < p; ++j) {
    double n1 = ctx->cnt_h[2 * j], n2 = ctx->cnt_h[2 * j + 1];
    double sq = n1 + 4.0 * n2, s = n1 + 2.0 * n2;
    const uint64_t ngi = n - (uint64_t)miss_h[j];
    double ng = (double)ngi;
    if (ngi > 1) {
      total_mean += s / ng;
      total_var += (sq - s * s / ng) / (ng - 1);
      ++nm;
      ++nv;
    } else if (ngi == 1) {
      total_mean += s / ng;
      ++nm;
    }
  }
  ctx->var_x = total_var / nv;
  ctx->mean_x = total_mean / nm;
  ctx->K.geno = g;
  ctx->K.cnt = cnt;
  ctx->have_geno = true;
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_set_phenotypes(bmg_ctx* ctx, const double* y, const uint8_t* mask, uint32_t n_pheno)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  if (!y || n_pheno == 0) throw bmg_error(BMG_EINVAL, "null phenotypes");
  const uint64_t n = ctx->n;
  if (n_pheno > 1 || mask) {
    // one chain per phenotype, each fitted to the individuals its mask keeps
    // (the reference runs one process per phenotype on a subset .bed)
    if (n_pheno != ctx->C)
      throw bmg_error(BMG_EUNSUPPORTED, "several phenotypes need one chain per phenotype (n_threads = phenotypes)");
    if (ctx->opt.m_e != 0) throw bmg_error(BMG_EUNSUPPORTED, "covariates are not supported with several phenotypes");
    if (ctx->opt.recode_g_to_minor_allele_count)
      throw bmg_error(BMG_EUNSUPPORTED, "the minor-allele recode would differ per sample; recode the .bed first");
    ctx->multi = true;
    ctx->ph_mask.assign((size_t)n_pheno * n, 1);
    if (mask)
      for (size_t q = 0; q < (size_t)n_pheno * n; ++q) ctx->ph_mask[q] = mask[q] ? 1 : 0;
    const uint32_t P = n_pheno;
    ctx->ph_n.assign(P, 0);
    ctx->ph_yy.assign(P, 0);
    ctx->ph_var_y.assign(P, 0);
    ctx->ph_amax.assign(P, 0);
    ctx->ph_ysum.assign(P, 0);
    ctx->ph_sy.assign(P, 0);
    std::vector<double> yall((size_t)P * n, 0.0);
    std::vector<int64_t> yint((size_t)P * n, 0);
    for (uint32_t k = 0; k < P; ++k) {
      const double* yk = y + (size_t)k * n;
      const uint8_t* mk = &ctx->ph_mask[(size_t)k * n];
      double cnt = 0, yy = 0, s = 0, amax = 0;
      for (uint64_t i = 0; i < n; ++i) {
        if (!mk[i]) continue;
        if (!std::isfinite(yk[i])) throw bmg_error(BMG_EINVAL, "non-finite phenotype");
        cnt += 1;
        yy += yk[i] * yk[i];
        s += yk[i];
        amax = std::max(amax, std::fabs(yk[i]));
        yall[(size_t)k * n + i] = yk[i];
      }
      if (cnt < 2) throw bmg_error(BMG_EINVAL, "a sample needs at least two individuals");
      ctx->ph_n[k] = cnt;
      ctx->ph_yy[k] = yy;
      ctx->ph_var_y[k] = (yy - s * s / cnt) / (cnt - 1);
      ctx->ph_amax[k] = amax;
      ctx->ph_ysum[k] = s;
      const int sy = fixed_exponent(amax, (uint64_t)cnt);
      ctx->ph_sy[k] = sy;
      for (uint64_t i = 0; i < n; ++i)
        if (mk[i]) yint[(size_t)k * n + i] = (int64_t)std::llrint(std::ldexp(yk[i], sy));
    }
    ctx->ph_y_dev = ctx->dalloc<double>((size_t)P * n, false);
    ctx->ph_yint_dev = ctx->dalloc<int64_t>((size_t)P * n, false);
    CK(cudaMemcpyAsync(ctx->ph_y_dev, yall.data(), 8 * yall.size(), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->ph_yint_dev, yint.data(), 8 * yint.size(), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    // the single-sample fields hold sample 0 (read by what reports one sample)
    ctx->y_h.assign(yall.begin(), yall.begin() + n);
    ctx->yy = ctx->ph_yy[0];
    ctx->var_y = ctx->ph_var_y[0];
    ctx->K.y = ctx->ph_y_dev;
    ctx->K.yint = ctx->ph_yint_dev;
    ctx->K.sy = ctx->ph_sy[0];
    ctx->K.y_absmax = ctx->ph_amax[0];
    ctx->have_y = true;
    return BMG_OK;
  }
  ctx->y_h.assign(y, y + n);
  double yy = 0, sq = 0, s = 0, amax = 0;
  for (uint64_t i = 0; i < n; ++i) {
    if (!std::isfinite(y[i])) throw bmg_error(BMG_EINVAL, "non-finite phenotype");
    yy += y[i] * y[i];
    amax = std::max(amax, std::fabs(y[i]));
  }
  for (uint64_t i = 0; i < n; ++i) { sq += y[i] * y[i]; s += y[i]; }
  ctx->yy = yy;
  ctx->var_y = (sq - s * s / n) / (n - 1);
  int sy = fixed_exponent(amax, n);
  std::vector<int64_t> yint(n);
  for (uint64_t i = 0; i < n; ++i) yint[i] = (int64_t)std::llrint(std::ldexp(y[i], sy));
  double* yd = ctx->dalloc<double>(n);
  int64_t* yi = ctx->dalloc<int64_t>(n);
  CK(cudaMemcpyAsync(yd, y, 8 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(yi, yint.data(), 8 * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->K.y = yd;
  ctx->K.yint = yi;
  ctx->K.sy = sy;
  ctx->K.y_absmax = amax;
  ctx->have_y = true;
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_set_covariates(bmg_ctx* ctx, const double* e, uint32_t m_e)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  if (m_e != ctx->opt.m_e) throw bmg_error(BMG_EINVAL, "m_e differs from the options");
  if (m_e > BMG_MAX_COV)
    throw bmg_error(BMG_EUNSUPPORTED, "at most " + std::to_string(BMG_MAX_COV) + " covariates on this path");
  if (m_e > 0 && !e) throw bmg_error(BMG_EINVAL, "null covariates");
  ctx->e_h.assign(e, e + (size_t)ctx->n * m_e);
  ctx->have_e = true;
  return BMG_OK;
  API_END
}

// The dd_add prefix of the chains that asked for it (all with force).
static void launch_rebuild(bmg_ctx* ctx, int force)
{
  const DevConst& K = ctx->K;
  dim3 grid((unsigned)((K.p + BMG_REBUILD_TILE - 1) / BMG_REBUILD_TILE), ctx->C);
  bmg_rebuild_sums_kernel<<<grid, 256, 0, ctx->stream>>>(K, force);
  LAUNCHED(ctx, "bmg_rebuild_sums_kernel");
  bmg_rebuild_write_kernel<<<grid, 256, 0, ctx->stream>>>(K);
  LAUNCHED(ctx, "bmg_rebuild_write_kernel");
}

// ------------------------------------------------------------- precompute

extern "C" bmg_status bmg_precompute(bmg_ctx* ctx)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  if (!ctx->have_geno || !ctx->have_y) throw bmg_error(BMG_EINVAL, "genotypes and phenotypes must be loaded first");
  if (ctx->opt.m_e > 0 && !ctx->have_e) throw bmg_error(BMG_EINVAL, "covariates must be set (m_e > 0)");
  const bmg_options& o = ctx->opt;
  const uint64_t n = ctx->n, p = ctx->p;
  const uint32_t C = ctx->C, km = ctx->km, me = o.m_e + 1;
  DevConst& K = ctx->K;
  K.n = n;
  K.p = p;
  K.gs = ctx->gs;
  K.nw = ctx->gs / 4;
  K.m_e = me;
  K.km = km;
  K.n_chains = C;
  K.n_types = o.n_types;
  int allow_types[5] = {0, 0, 0, 0, 0}, allow_terms[4] = {0, 0, 0, 0};
  for (uint32_t t = 0; t < o.n_types; ++t) {
    K.types[t] = o.types[t];
    allow_types[o.types[t]] = 1;
    if (o.types[t] == BMG_TYPE_AH) { allow_terms[0] = allow_terms[1] = 1; }
    else allow_terms[o.types[t]] = 1;
  }
  for (int t = 0; t < 5; ++t) K.allow_types[t] = allow_types[t];
  for (int t = 0; t < 4; ++t) K.allow_terms[t] = allow_terms[t];
  /* src/precomputed_snp_covariances.hpp:58-84 */
  bool ah = allow_types[4], a = allow_types[0], h = allow_types[1];
  int offset = 2 * (int)o.n_types + (ah ? 1 : 0) * (1 + ((a && h) ? -2 : 0) + ((a || h) ? 0 : 2));
  K.offset = offset;
  int oi = 0;
  K.n_terms = 0;
  for (int t = 0; t < 4; ++t) {
    K.offset_type[t] = allow_terms[t] ? oi++ : -1;
    if (allow_terms[t]) K.term_of[K.n_terms++] = t;
  }
  // per-SNP sums and centred second moments from the counts (exact integers)
  ctx->pre_h.assign(p * offset, 0.0);
  for (uint64_t j = 0; j < p; ++j) {
    double n1 = ctx->cnt_h[2 * j], n2 = ctx->cnt_h[2 * j + 1];
    double* loc = &ctx->pre_h[j * offset];
    for (int t = 0; t < 4; ++t) {
      if (!allow_terms[t]) continue;
      double ch_ = (t == 3) ? 0 : 1, cr = (t == 0) ? 2 : (t == 1 ? 0 : 1);
      double xs = ch_ * n1 + cr * n2;
      double xx = ch_ * ch_ * n1 + cr * cr * n2;
      *loc++ = xs;
      *loc++ = xx - xs * xs / (double)n;
    }
    if (ah) {
      double as = n1 + 2 * n2, hs = n1;
      *loc++ = n1 - as * hs / (double)n;
    }
  }
  double* pre = ctx->dalloc<double>(p * offset, false);
  CK(cudaMemcpyAsync(pre, ctx->pre_h.data(), 8 * p * offset, cudaMemcpyHostToDevice, ctx->stream));
  K.pre = pre;
  K.lvar = nullptr;
  // in-order ranks of the proposal tree
  std::vector<int32_t> pos, inv;
  inorder_ranks(p, pos, inv);
  int32_t* dpos = ctx->dalloc<int32_t>(p, false);
  int32_t* dinv = ctx->dalloc<int32_t>(p, false);
  CK(cudaMemcpyAsync(dpos, pos.data(), 4 * p, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(dinv, inv.data(), 4 * p, cudaMemcpyHostToDevice, ctx->stream));
  K.pos = dpos;
  K.inv = dinv;
  // covariates with the constant column (src/data.hpp:48,53)
  std::vector<double> E((size_t)n * me, 1.0);
  for (uint32_t j = 1; j < me; ++j)
    for (uint64_t i = 0; i < n; ++i) E[(size_t)j * n + i] = ctx->e_h[(size_t)(j - 1) * n + i];
  std::vector<double> ee((size_t)me * me, 0.0), ey(me, 0.0), emax(me, 1.0);
  for (uint32_t j = 0; j < me; ++j)
    for (uint32_t i = 0; i <= j; ++i) {
      double t = 0;
      for (uint64_t l = 0; l < n; ++l) t += E[(size_t)i * n + l] * E[(size_t)j * n + l];
      ee[(size_t)j * me + i] = t;
    }
  for (uint32_t j = 0; j < me; ++j) {
    double t = 0;
    for (uint64_t l = 0; l < n; ++l) t += E[(size_t)j * n + l] * ctx->y_h[l];
    ey[j] = t;
  }
  std::vector<int64_t> eint((size_t)n * me, 0);
  std::vector<int32_t> se(me, 0);
  for (uint32_t j = 1; j < me; ++j) {
    double am = 0;
    for (uint64_t l = 0; l < n; ++l) am = std::max(am, std::fabs(E[(size_t)j * n + l]));
    emax[j] = am;
    se[j] = fixed_exponent(am, n);
    for (uint64_t l = 0; l < n; ++l) eint[(size_t)j * n + l] = (int64_t)std::llrint(std::ldexp(E[(size_t)j * n + l], se[j]));
  }
  double* dE = ctx->dalloc<double>(E.size(), false);
  int64_t* dEi = ctx->dalloc<int64_t>(eint.size(), false);
  int32_t* dse = ctx->dalloc<int32_t>(me, false);
  double* dee = ctx->dalloc<double>(ee.size(), false);
  double* dey = ctx->dalloc<double>(me, false);
  double* demax = ctx->dalloc<double>(me, false);
  std::vector<double> ite(me, o.inv_tau2_e_val);
  ite[0] = o.inv_tau2_e_const_val;
  double* dite = ctx->dalloc<double>(me, false);
  CK(cudaMemcpyAsync(dE, E.data(), 8 * E.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(dEi, eint.data(), 8 * eint.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(dse, se.data(), 4 * me, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(dee, ee.data(), 8 * ee.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(dey, ey.data(), 8 * me, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(demax, emax.data(), 8 * me, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(dite, ite.data(), 8 * me, cudaMemcpyHostToDevice, ctx->stream));
  K.e = dE;
  K.eint = dEi;
  K.se = dse;
  {
    // X'y and X'E of every SNP and term, from exact per-SNP H/R sums
    const uint32_t nv = std::max<uint32_t>(1, me);
    int64_t* gsum = ctx->dalloc<int64_t>((size_t)K.p * nv * 2, false);
    const uint64_t blocks = std::min<uint64_t>((K.p + 7) / 8, 152 * 8);
    bmg_gsum_kernel<<<(unsigned)blocks, 256, 0, ctx->stream>>>(K.geno, n, K.p, K.gs, K.yint, dEi, nv, gsum);
    LAUNCHED(ctx, "bmg_gsum_kernel");
    K.gsum = gsum;
  }
  K.ee = dee;
  K.ey = dey;
  K.e_absmax = demax;
  K.inv_tau2_e = dite;
  K.yy = ctx->yy;
  /* src/sampler.hpp:173-199 */
  double s2s = (o.s2_sigma2 > 0) ? o.s2_sigma2
                                 : ctx->var_y * (1 - o.R2mode_sigma2) * (o.nu_sigma2 + 2) / o.nu_sigma2;
  ctx->s2_sigma2 = s2s;
  double s2t[4] = {0, 0, 0, 0};
  for (int t = 0; t < 4; ++t) {
    if (!allow_terms[t]) continue;
    if (o.s2_tau2[t] > 0) s2t[t] = o.s2_tau2[t];
    else
      s2t[t] = o.eh_tau2[t] * (o.nu_tau2[t] - 2) /
               (o.nu_tau2[t] * (ctx->var_x + ctx->mean_x * ctx->mean_x) * (1 - o.R2mode_sigma2));
    ctx->s2_tau2[t] = s2t[t];
  }
  /* src/prior.hpp:45-122 */
  if (s2s <= 0)
    throw bmg_error(BMG_EINVAL, "Prior specification error: s2_sigma2 is not positive (Probably option s2_sigma2 is "
                                "not specified and using R2mode_sigma2 leads to the invalid value).");
  if (o.nu_sigma2 < 0) throw bmg_error(BMG_EINVAL, "Prior specification error: nu_sigma2 is negative.");
  double ga, gb;
  {
    double eq = o.e_qg, vq = o.var_qg;
    if (p > 1) {
      double z = (vq - eq * (1 - eq)) / ((p - 1) * eq);
      ga = (z - 1) / (1 - p * z / eq);
      gb = (p / eq - 1) * ga;
    } else {
      double z = eq / (1 - eq);
      gb = z / vq / std::pow(1 + z, 3) - 1 / (1 + z);
      ga = z * gb;
    }
    if (ga <= 0 || gb <= 0 || std::isnan(ga) || std::isnan(gb)) throw bmg_error(BMG_EINVAL, "Invalid a or b.");
  }
  ctx->g_a = ga;
  ctx->g_b = gb;
  K.g_a = ga;
  K.g_b = gb;
  double tps = 0;
  for (int t = 0; t < 5; ++t) {
    K.types_prior[t] = allow_types[t] ? o.types_prior[t] : NAN;
    if (allow_types[t]) tps += o.types_prior[t];
  }
  K.types_prior_sum = tps;
  double alpha0 = std::max(0.5, o.mu_alpha), alpha2 = alpha0 * alpha0;
  double inv0[4];
  for (int t = 0; t < 4; ++t) {
    if (allow_terms[t]) {
      if (s2t[t] <= 0)
        throw bmg_error(BMG_EINVAL, std::string("Prior specification error: s2_tau2 for ") + kTypeName[t] +
                                        " is not positive.");
      if (o.nu_tau2[t] <= 0)
        throw bmg_error(BMG_EINVAL, std::string("Prior specification error: nu_tau2 for ") + kTypeName[t] +
                                        " is not positive.");
      K.nu_tau2[t] = o.nu_tau2[t];
      K.s2_tau2[t] = s2t[t];
      K.nus2_tau2[t] = o.nu_tau2[t] * s2t[t];
      double tau2_init = K.nus2_tau2[t] / std::max(0.1, (o.nu_tau2[t] - 2));
      inv0[t] = 1.0 / (alpha2 * tau2_init);
    } else {
      K.nu_tau2[t] = K.s2_tau2[t] = K.nus2_tau2[t] = NAN;
      inv0[t] = NAN;
    }
  }
  K.n_plus_nu = (double)n + o.nu_sigma2;
  K.minus_n_plus_nu_2 = -0.5 * K.n_plus_nu;
  K.nus2_plus_yy = o.nu_sigma2 * s2s + ctx->yy;
  // the samples the chains are fitted to: one record for all chains, or one
  // per phenotype; per chain the covariate block and the initial precisions
  std::vector<DevPheno> recs;
  std::vector<uint32_t> pheno_of(C, 0);
  std::vector<double> chain_ee0(C, ee[0]), chain_ey0(C, ey[0]);
  std::vector<std::array<double, 4>> chain_inv0(C);
  for (uint32_t c = 0; c < C; ++c)
    for (int t = 0; t < 4; ++t) chain_inv0[c][t] = inv0[t];
  if (!ctx->multi) {
    DevPheno r;
    std::memset(&r, 0, sizeof(r));
    r.n = (double)n;
    r.n_plus_nu = K.n_plus_nu;
    r.minus_n_plus_nu_2 = K.minus_n_plus_nu_2;
    r.nus2_plus_yy = K.nus2_plus_yy;
    r.rng_nu = (double)n + o.nu_sigma2;
    for (int t = 0; t < 4; ++t) r.nus2_tau2[t] = K.nus2_tau2[t];
    r.y_absmax = K.y_absmax;
    r.sy = K.sy;
    r.y = K.y;
    r.yint = K.yint;
    r.mask2 = nullptr;
    r.cnt = K.cnt;
    r.pre = K.pre;
    r.gsum = K.gsum;
    recs.push_back(r);
  } else {
    const uint32_t P = C;
    const size_t nw64 = ctx->gs / 8;
    std::vector<uint64_t> m2((size_t)P * nw64, 0);
    for (uint32_t k = 0; k < P; ++k)
      for (uint64_t i = 0; i < n; ++i)
        if (ctx->ph_mask[(size_t)k * n + i]) m2[(size_t)k * nw64 + (i >> 5)] |= 1ull << (2 * (i & 31));
    uint64_t* dm2 = ctx->dalloc<uint64_t>(m2.size(), false);
    int32_t* dcnt = ctx->dalloc<int32_t>((size_t)P * p * 2, false);
    double* dpre = ctx->dalloc<double>((size_t)P * p * offset, false);
    double* dn = ctx->dalloc<double>(P, false);
    CK(cudaMemcpyAsync(dm2, m2.data(), 8 * m2.size(), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(dn, ctx->ph_n.data(), 8 * P, cudaMemcpyHostToDevice, ctx->stream));
    const uint64_t warps = (uint64_t)P * p;
    bmg_mask_counts_kernel<<<(unsigned)std::min<uint64_t>((warps + 7) / 8, 152 * 16), 256, 0, ctx->stream>>>(
        K.geno, ctx->gs, p, dm2, P, dcnt);
    LAUNCHED(ctx, "bmg_mask_counts_kernel");
    int amask = 0;
    for (int t = 0; t < 4; ++t) amask |= allow_terms[t] ? (1 << t) : 0;
    bmg_pre_kernel<<<1024, 256, 0, ctx->stream>>>(dcnt, p, P, dn, amask, ah ? 1 : 0, offset, dpre);
    LAUNCHED(ctx, "bmg_pre_kernel");
    // var_x and mean_x of a sample (src/data.cpp:403-434) enter only where the
    // term precision's scale comes from eh_tau2
    bool need_x = false;
    for (int t = 0; t < 4; ++t) need_x = need_x || (allow_terms[t] && !(o.s2_tau2[t] > 0));
    std::vector<int32_t> hc;
    if (need_x) {
      hc.resize((size_t)P * p * 2);
      CK(cudaMemcpyAsync(hc.data(), dcnt, 4 * hc.size(), cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    for (uint32_t k = 0; k < P; ++k) {
      const double nk = ctx->ph_n[k];
      double vx = 0, mx = 0;
      if (need_x) {
        double tv = 0, tm = 0;
        for (uint64_t j = 0; j < p; ++j) {
          const double n1 = hc[((size_t)k * p + j) * 2], n2 = hc[((size_t)k * p + j) * 2 + 1];
          const double sq = n1 + 4.0 * n2, sm = n1 + 2.0 * n2;
          tm += sm / nk;
          tv += (sq - sm * sm / nk) / (nk - 1);
        }
        vx = tv / p;
        mx = tm / p;
      }
      const double s2s_k = (o.s2_sigma2 > 0) ? o.s2_sigma2
                                             : ctx->ph_var_y[k] * (1 - o.R2mode_sigma2) * (o.nu_sigma2 + 2) / o.nu_sigma2;
      if (s2s_k <= 0) throw bmg_error(BMG_EINVAL, "Prior specification error: s2_sigma2 is not positive (sample " +
                                                      std::to_string(k) + ")");
      DevPheno r;
      std::memset(&r, 0, sizeof(r));
      r.n = nk;
      r.n_plus_nu = nk + o.nu_sigma2;
      r.minus_n_plus_nu_2 = -0.5 * r.n_plus_nu;
      r.nus2_plus_yy = o.nu_sigma2 * s2s_k + ctx->ph_yy[k];
      r.rng_nu = nk + o.nu_sigma2;
      for (int t = 0; t < 4; ++t) {
        if (!allow_terms[t]) {
          r.nus2_tau2[t] = NAN;
          chain_inv0[k][t] = NAN;
          continue;
        }
        const double s2t_k = (o.s2_tau2[t] > 0) ? o.s2_tau2[t]
                                                : o.eh_tau2[t] * (o.nu_tau2[t] - 2) /
                                                      (o.nu_tau2[t] * (vx + mx * mx) * (1 - o.R2mode_sigma2));
        if (!(s2t_k > 0)) throw bmg_error(BMG_EINVAL, "Prior specification error: s2_tau2 is not positive");
        r.nus2_tau2[t] = o.nu_tau2[t] * s2t_k;
        chain_inv0[k][t] = 1.0 / (alpha2 * (r.nus2_tau2[t] / std::max(0.1, (o.nu_tau2[t] - 2))));
      }
      r.y_absmax = ctx->ph_amax[k];
      r.sy = ctx->ph_sy[k];
      r.y = ctx->ph_y_dev + (size_t)k * n;
      r.yint = ctx->ph_yint_dev + (size_t)k * n;
      r.mask2 = dm2 + (size_t)k * nw64;
      r.cnt = dcnt + (size_t)k * p * 2;
      r.pre = dpre + (size_t)k * p * offset;
      r.gsum = nullptr;
      recs.push_back(r);
      pheno_of[k] = k;
      chain_ee0[k] = nk;
      chain_ey0[k] = ctx->ph_ysum[k];
    }
  }
  // one-type scans evaluate the posterior in double-float from FP32 copies
  // of the two sums it reads
  if (o.n_types == 1 && o.types[0] != 4 && !o.use_individual_tau2) {
    const uint32_t off = (uint32_t)K.offset_type[o.types[0]];
    for (DevPheno& r : recs) {
      float4* pf = ctx->dalloc<float4>(p, false);
      bmg_pre_df_kernel<<<1024, 256, 0, ctx->stream>>>(r.pre, p, (uint32_t)offset, off, pf);
      LAUNCHED(ctx, "bmg_pre_df_kernel");
      r.pre_f = pf;
    }
  }
  {
    DevPheno* dph = ctx->dalloc<DevPheno>(recs.size(), false);
    uint32_t* dpo = ctx->dalloc<uint32_t>(C, false);
    CK(cudaMemcpyAsync(dph, recs.data(), sizeof(DevPheno) * recs.size(), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(dpo, pheno_of.data(), 4 * C, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    K.ph = dph;
    K.pheno_of = dpo;
  }
  K.mu_alpha = o.mu_alpha;
  K.use_individual_tau2 = o.use_individual_tau2;
  K.rng_nu = (double)n + o.nu_sigma2;
  K.n_rao = o.n_rao;
  K.thin = o.thin;
  K.n_sample_tau2 = o.n_sample_tau2_and_missing;
  K.verbosity = o.verbosity;
  K.max_move_size = (uint32_t)ctx->max_ms;
  K.max_nbh = o.max_SNP_neighborhood_size;
  K.p_move_size_nbs = o.p_move_size_nbs;
  K.p_move_size_nbc = o.p_move_size_nbc;
  K.adapt_p_move_size = o.adapt_p_move_size && ctx->max_ms > 1;
  K.acpt_goal = o.p_move_size_acpt_goal;
  K.adaptation = o.adaptation;
  K.flat_proposal_dist = o.flat_proposal_dist;
  K.save_beta = o.save_beta;
  K.q_add_min = 1.0 / (p - o.e_qg);
  K.q_rem_min = 1.0 / o.e_qg;
  // prior tables, evaluated with the reference's expressions (src/prior.hpp:144-183)
  const uint32_t tw = km + 2;
  K.tw = tw;
  std::vector<double> tab((size_t)22 * tw, 0.0);
  auto T = [&](int which, uint32_t k) -> double& { return tab[(size_t)which * tw + k]; };
  const double mg = (double)p;
  for (uint32_t k = 0; k < tw; ++k) {
    int nl = (int)k;
    T(0, k) = std::log(ga + nl) - std::log(gb + p - nl - 1);
    T(1, k) = std::log(gb + p - nl) - std::log(ga + nl - 1);
    for (int t = 0; t < 5; ++t) {
      double tp = K.types_prior[t];
      T(2 + t, k) = std::log(tp + nl);
      T(7 + t, k) = std::log(tp + nl - 1);
      T(14 + t, k) = std::lgamma(tp + (double)nl);
    }
    T(12, k) = std::log(tps + nl);
    T(13, k) = std::log(tps + nl - 1);
    T(19, k) = std::lgamma(ga + (double)nl);
    T(20, k) = std::lgamma(gb + mg - (double)nl);
    T(21, k) = std::lgamma(tps + (double)nl);
  }
  double* dtab = ctx->dalloc<double>(tab.size(), false);
  CK(cudaMemcpyAsync(dtab, tab.data(), 8 * tab.size(), cudaMemcpyHostToDevice, ctx->stream));
  K.tab = dtab;
  {  // the move-size grid of Sampler::adapt_p_move_size_jd_mb (src/sampler.hpp:1739-1766)
    std::vector<double> grid(50), pw(51);
    double pp = 0.01, step = 0.98 / 49.0;
    for (int j = 0; j < 50; ++j) {
      grid[j] = pp;
      pw[j] = std::pow(1 - pp, (double)ctx->max_ms);
      pp += step;
    }
    pw[50] = std::pow(1 - o.p_move_size, (double)ctx->max_ms);
    double* dg = ctx->dalloc<double>(50, false);
    double* dp = ctx->dalloc<double>(51, false);
    CK(cudaMemcpyAsync(dg, grid.data(), 8 * 50, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(dp, pw.data(), 8 * 51, cudaMemcpyHostToDevice, ctx->stream));
    K.ms_grid = dg;
    K.ms_pow = dp;
    K.ms_init = o.p_move_size;
  }
  int qbits = 0;
  while ((1ull << qbits) < p + 1) ++qbits;
  K.qs = 61 - qbits;
  // per-chain state
  K.cur = ctx->dalloc<DevModel>(C);
  K.nm = ctx->dalloc<DevModel>(C);
  K.ch = ctx->dalloc<DevChain>(C);
  K.rb = ctx->dalloc<RbParams>(C);
  const size_t pc = (size_t)p * C;
  K.p_prop = ctx->dalloc<double>(pc, false);
  K.p_prop_types = ctx->dalloc<double>(o.n_types > 1 ? pc * o.n_types : 1, false);
  K.p_rao = ctx->dalloc<double>(pc);
  K.p_rao_types = ctx->dalloc<double>(o.n_types > 1 ? pc * o.n_types : 1);
  K.p_r = ctx->dalloc<double>(pc);
  K.p_r_types = ctx->dalloc<double>(o.n_types > 1 ? pc * o.n_types : 1);
  K.q_ms = ctx->dalloc<double>((size_t)C * 256);
  K.q_nbs = ctx->dalloc<double>((size_t)C * 128);
  K.q_nbc = ctx->dalloc<double>((size_t)C * 256);
  K.r_ms_sum = ctx->dalloc<double>((size_t)C * 256);
  K.r_ms_n = ctx->dalloc<double>((size_t)C * 256);
  K.q_p0_ms = ctx->dalloc<double>((size_t)C * 256);
  K.cadd = ctx->dalloc<int64_t>((size_t)(p + 1) * C);
  const size_t words = (p + 31) / 32;
  K.inbits = ctx->dalloc<uint32_t>(words * C);
  K.basebits = ctx->dalloc<uint32_t>(words * C);
  K.tile_sums = ctx->dalloc<int64_t>((size_t)C * ((p + BMG_REBUILD_TILE - 1) / BMG_REBUILD_TILE));
  K.rebuild_active = ctx->dalloc<int32_t>(C);
  // learned proposal: candidate tables, features, MLP parameters
  K.lrn.on = o.proposal == BMG_PROPOSAL_LEARNED;
  if (K.lrn.on) {
    DevLearned& L = K.lrn;
    L.mix = o.learned_mix;
    L.topk = o.learned_topk;
    L.t_snp = ctx->dalloc<uint32_t>((size_t)C * L.topk);
    L.t_s = ctx->dalloc<double>((size_t)C * L.topk);
    L.t_sum = ctx->dalloc<double>(C);
    L.t_n = ctx->dalloc<uint32_t>(C);
    L.maxcorr = ctx->dalloc<float>((size_t)C * p);
    L.logit = ctx->dalloc<float>((size_t)C * p);
    L.theta = ctx->dalloc<float>(MLP_NPAR);
    L.grad = ctx->dalloc<float>(MLP_NPAR);
    L.adam_m = ctx->dalloc<float>(MLP_NPAR);
    L.adam_v = ctx->dalloc<float>(MLP_NPAR);
    L.w1b = ctx->dalloc<uint16_t>(MLP_H * MLP_F);
    L.w2b = ctx->dalloc<uint16_t>(MLP_H * MLP_H);
    ctx->adam_t = ctx->dalloc<int32_t>(1);
    // the scans keep the per-SNP log odds, the first feature
    if (!ctx->lml_buf) ctx->lml_buf = ctx->dalloc<double>((size_t)C * p);
    K.p_lml = ctx->lml_buf;
    CK(bmg_mlp_init(&K, ctx->adam_t, ctx->stream));
  }
  K.model_inds = ctx->dalloc<int32_t>(pc, false);
  CK(cudaMemsetAsync(K.model_inds, 0xff, 4 * pc, ctx->stream));
  K.n_pad = ctx->n_pad;
  K.limbs_n = ctx->L;
  K.wait_limit = ctx->wait_limit;
  K.resid = ctx->dalloc<int64_t>((size_t)C * ctx->n_pad);
  K.yhat = ctx->dalloc<double>((size_t)C * n);
  K.limbs = ctx->dalloc<uint16_t>((size_t)C * ctx->L * ctx->n_pad);
  ctx->resid_t = ctx->dalloc<int64_t>((size_t)C * ctx->n_pad);
  K.scratch = ctx->dalloc<double>((size_t)C * 2 * km);
  // missing calls: the CSR, the imputation prior and every chain's values
  // (all 0 at the start, as the reference's DataModel starts them)
  K.miss_total = ctx->miss_ind.size();
  K.miss_snps = 0;
  if (K.miss_total) {
    if (ctx->multi) throw bmg_error(BMG_EUNSUPPORTED, "missing genotype calls with several phenotypes are not on this path");
    std::vector<int32_t> rank(p, -1);
    std::vector<uint32_t> list;
    for (uint64_t j = 0; j < p; ++j)
      if (ctx->miss_off[j + 1] > ctx->miss_off[j]) {
        rank[j] = (int32_t)list.size();
        list.push_back((uint32_t)j);
      }
    K.miss_snps = (uint32_t)list.size();
    int64_t* off = ctx->dalloc<int64_t>(p + 1, false);
    uint32_t* ind = ctx->dalloc<uint32_t>(K.miss_total, false);
    double* pri = ctx->dalloc<double>(3 * p, false);
    int32_t* rk = ctx->dalloc<int32_t>(p, false);
    uint32_t* ls = ctx->dalloc<uint32_t>(list.size(), false);
    CK(cudaMemcpyAsync(off, ctx->miss_off.data(), 8 * (p + 1), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ind, ctx->miss_ind.data(), 4 * K.miss_total, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(pri, ctx->miss_prior.data(), 8 * 3 * p, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(rk, rank.data(), 4 * p, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ls, list.data(), 4 * list.size(), cudaMemcpyHostToDevice, ctx->stream));
    K.miss_off = off;
    K.miss_ind = ind;
    K.miss_prior = pri;
    K.miss_rank = rk;
    K.miss_list = ls;
    K.miss_val = ctx->dalloc<uint8_t>((size_t)C * K.miss_total);
    K.miss_corr = ctx->dalloc<MissCorr>((size_t)C * list.size());
    K.miss_fit = ctx->dalloc<long long>((size_t)C * ctx->n_pad);
    K.miss_yh = ctx->dalloc<double>((size_t)C * n);
    K.miss_inm = ctx->dalloc<long long>((size_t)C * 2 * km);
  }
  K.dr = ctx->dr;
  if (ctx->dr) {
    K.dr_l = ctx->dalloc<double>((size_t)C * km * (km + 1) / 2);
    K.dr_v = ctx->dalloc<double>((size_t)C * km);
    K.dr_inv = ctx->dalloc<double>((size_t)C * km);
    K.dr_ti = ctx->dalloc<uint8_t>((size_t)C * km);
    K.dr_x1 = ctx->dalloc<uint32_t>((size_t)C * km);
    K.dr_x2 = ctx->dalloc<uint32_t>((size_t)C * km);
    K.dr_pm = ctx->dalloc<double>((size_t)C << ctx->dr);
  }
  // trace buffers of one chunk
  uint32_t gi = o.graph_iters ? o.graph_iters : 64;
  ctx->opt.graph_iters = gi;
  DevTrace& tr = K.tr;
  tr.iter_cap = gi;
  tr.thin_cap = (uint32_t)(gi / o.thin + 2);
  tr.loci_cap = tr.thin_cap * km;
  tr.beta_cap = o.save_beta ? tr.thin_cap * km : 1;
  tr.log_cap = o.verbosity ? (uint32_t)(gi / o.verbosity + 2) : 1;
  tr.jump = ctx->dalloc<uint8_t>((size_t)C * tr.iter_cap);
  tr.mtype = ctx->dalloc<uint8_t>((size_t)C * tr.iter_cap);
  tr.msize = ctx->dalloc<uint8_t>((size_t)C * tr.iter_cap);
  tr.msz = ctx->dalloc<uint32_t>((size_t)C * tr.thin_cap);
  tr.loci = ctx->dalloc<uint32_t>((size_t)C * tr.loci_cap);
  tr.types = ctx->dalloc<uint8_t>((size_t)C * tr.loci_cap);
  tr.ll = ctx->dalloc<double>((size_t)C * tr.thin_cap);
  tr.lp = ctx->dalloc<double>((size_t)C * tr.thin_cap);
  tr.s2 = ctx->dalloc<double>((size_t)C * tr.thin_cap);
  tr.alpha = ctx->dalloc<double>((size_t)C * tr.thin_cap);
  tr.pve = ctx->dalloc<double>((size_t)C * tr.thin_cap * 3);
  tr.beta = ctx->dalloc<double>((size_t)C * tr.beta_cap);
  tr.logrec = ctx->dalloc<double>((size_t)C * tr.log_cap * BMG_LOGREC);
  // models and chains
  std::vector<DevModel> models(2 * C);
  for (uint32_t c = 0; c < 2 * C; ++c) {
    DevModel& M = models[c];
    std::memset(&M, 0, sizeof(M));
    M.xx = ctx->dalloc<double>((size_t)km * km);
    M.l = ctx->dalloc<double>((size_t)km * (km + 1) / 2);  // packed upper triangle
    M.xy = ctx->dalloc<double>(km);
    M.v = ctx->dalloc<double>(km);
    M.inv = ctx->dalloc<double>(km);
    M.beta = ctx->dalloc<double>(km);
    M.mu_beta = ctx->dalloc<double>(km);
    M.loci = ctx->dalloc<uint32_t>(km);
    M.type_inds = ctx->dalloc<uint8_t>(km);
    M.x_ind1 = ctx->dalloc<uint32_t>(km);
    M.x_ind2 = ctx->dalloc<uint32_t>(km);
    M.xc_snp = ctx->dalloc<uint32_t>(km);
    M.xc_type = ctx->dalloc<int32_t>(km);
    M.xcols = (int)me;
    M.llen = M.vlen = M.blen = (int)me;
    M.ll = NAN;
    // covariate block (src/model.hpp:92-105)
    std::vector<double> xx((size_t)me * km, 0.0), xy0(ey);
    for (uint32_t j = 0; j < me; ++j)
      for (uint32_t i = 0; i <= j; ++i) xx[(size_t)j * km + i] = ee[(size_t)j * me + i];
    if (ctx->multi) {  // the constant column of this chain's sample
      xx[0] = chain_ee0[c % C];
      xy0[0] = chain_ey0[c % C];
    }
    CK(cudaMemcpyAsync(M.xx, xx.data(), 8 * xx.size(), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(M.xy, xy0.data(), 8 * me, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(M.inv, ite.data(), 8 * me, cudaMemcpyHostToDevice, ctx->stream));
    std::vector<int32_t> xt(me, 4);
    CK(cudaMemcpyAsync(M.xc_type, xt.data(), 4 * me, cudaMemcpyHostToDevice, ctx->stream));
  }
  CK(cudaMemcpyAsync(K.cur, models.data(), sizeof(DevModel) * C, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(K.nm, models.data() + C, sizeof(DevModel) * C, cudaMemcpyHostToDevice, ctx->stream));
  std::vector<DevChain> chs(C);
  std::vector<double> qms((size_t)C * 256, 0.0), qnbs((size_t)C * 128, 0.0), qnbc((size_t)C * 256, 0.0);
  const int mm2 = (ctx->max_ms + 1) / 2;
  for (uint32_t c = 0; c < C; ++c) {
    DevChain& h = chs[c];
    std::memset(&h, 0, sizeof(h));
    bmg_rng_init(&h.rng, ctx->seeds[c]);
    h.n_rao_burnin = o.n_rao_burnin;
    h.p_proposal_n = 1;
    h.p_rao_n = 0;
    h.n_moves[0] = h.n_moves[1] = h.n_moves[2] = 2;
    h.n_acpt[0] = h.n_acpt[1] = h.n_acpt[2] = 1;
    h.alpha = alpha0;
    h.alpha2 = alpha2;
    for (int t = 0; t < 4; ++t) h.inv_t2a2[t] = chain_inv0[c][t];
    h.p_move_size = o.p_move_size;
    h.k_move_size = 1000.0 / (double)o.n_rao_burnin;
    geometric_cdf(ctx->max_ms, o.p_move_size, &qms[(size_t)c * 256]);
    geometric_cdf(mm2, o.p_move_size_nbs, &qnbs[(size_t)c * 128]);
    geometric_cdf(ctx->max_ms, o.p_move_size_nbc, &qnbc[(size_t)c * 256]);
  }
  CK(cudaMemcpyAsync(K.ch, chs.data(), sizeof(DevChain) * C, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(K.q_ms, qms.data(), 8 * qms.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(K.q_nbs, qnbs.data(), 8 * qnbs.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(K.q_nbc, qnbc.data(), 8 * qnbc.size(), cudaMemcpyHostToDevice, ctx->stream));
  /* src/sampler.hpp:351-362 */
  double val = (ga / (ga + gb) * p) / (double)p;
  std::vector<double> flat(pc, val);
  CK(cudaMemcpyAsync(K.p_prop, flat.data(), 8 * pc, cudaMemcpyHostToDevice, ctx->stream));
  if (o.n_types > 1) {
    std::vector<double> ft(pc * o.n_types, 1.0 / o.n_types);
    CK(cudaMemcpyAsync(K.p_prop_types, ft.data(), 8 * ft.size(), cudaMemcpyHostToDevice, ctx->stream));
  }
  CK(bmg_move_configure(&ctx->move_smem));
  bmg_init_kernel<<<C, 32, ctx->move_smem, ctx->stream>>>(K);
  LAUNCHED(ctx, "bmg_init_kernel");
  launch_rebuild(ctx, 1);
  CK(cudaStreamSynchronize(ctx->stream));
  device_error_check(ctx);
  ctx->ready = true;
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_get_precomputed(bmg_ctx* ctx, double* xx, uint32_t* offset)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  if (offset) *offset = (uint32_t)ctx->K.offset;
  if (xx) std::memcpy(xx, ctx->pre_h.data(), 8 * ctx->pre_h.size());
  return BMG_OK;
  API_END
}

// ------------------------------------------------------------------- run

static void launch_scan(bmg_ctx* ctx)
{
  DevConst& K = ctx->K;
  if (K.miss_total) {
    // the missing calls' part of the scan (imputation outside the model)
    dim3 g((K.miss_snps + 7) / 8, ctx->C);
    bmg_miss_scan_kernel<<<g, 256, 0, ctx->stream>>>(K);
    LAUNCHED(ctx, "bmg_miss_scan_kernel");
  }
  bool tc = ctx->opt.scan_impl == BMG_SCAN_TCGEN05 && bmg_scan_tc_supported(&K);
  if (tc) {
    int v = ctx->tc_forced >= 0 ? ctx->tc_forced : ctx->tc_variant;
    const int nv = bmg_scan_tc_variants();
    if (v < 0) {
      // read the previous tuning scan, then time the next shape
      // every shape is timed twice (the fastest of the two counts) after one
      // warm-up scan
      if (ctx->tc_pending >= 0) {
        float ms = 0;
        CK(cudaEventSynchronize(ctx->tc_ev[1]));
        CK(cudaEventElapsedTime(&ms, ctx->tc_ev[0], ctx->tc_ev[1]));
        float& slot = ctx->tc_ms[ctx->tc_pending];
        if (ctx->tc_tuned > 1 && (slot < 0 || ms < slot)) slot = ms;
        ctx->tc_pending = -1;
      }
      if (ctx->tc_ms.empty()) {
        ctx->tc_ms.assign(nv, -1.0f);
        // shapes whose plan repeats an earlier shape's are not timed
        ctx->tc_cands.clear();
        for (int i = 0; i < nv; ++i)
          if (!bmg_scan_tc_variant_redundant(&K, i)) ctx->tc_cands.push_back(i);
      }
      const int nc = (int)ctx->tc_cands.size();
      if (ctx->tc_tuned > 2 * nc) {
        int best = ctx->tc_cands[0];
        for (int i : ctx->tc_cands)
          if (ctx->tc_ms[i] >= 0 && (ctx->tc_ms[best] < 0 || ctx->tc_ms[i] < ctx->tc_ms[best])) best = i;
        ctx->tc_variant = v = best;
      } else {
        v = ctx->tc_cands[ctx->tc_tuned == 0 ? 0 : (ctx->tc_tuned - 1) % nc];
        ctx->tc_pending = v;
        ++ctx->tc_tuned;
        for (int q = 0; q < 2; ++q)
          if (!ctx->tc_ev[q]) CK(cudaEventCreate(&ctx->tc_ev[q]));
        CK(cudaEventRecord(ctx->tc_ev[0], ctx->stream));
      }
    }
    int rc = bmg_scan_tc_launch(&K, ctx->stream, v);
    if (ctx->tc_pending >= 0 && rc == 0) CK(cudaEventRecord(ctx->tc_ev[1], ctx->stream));
    if (rc != 0)
      throw bmg_error(BMG_ECUDA, "tensor-core scan launch failed (step " + std::to_string(rc) +
                                     "): " + cudaGetErrorString(cudaGetLastError()));
    LAUNCHED(ctx, "bmg_scan_tc_kernel");
  } else {
    bmg_resid_transpose_kernel<<<1024, 256, 0, ctx->stream>>>(K, ctx->resid_t);
    LAUNCHED(ctx, "bmg_resid_transpose_kernel");
    unsigned blocks = 152 * 8;
    bmg_scan_simt_kernel<<<blocks, 256, 0, ctx->stream>>>(K, ctx->resid_t);
    LAUNCHED(ctx, "bmg_scan_simt_kernel");
  }
}

static void open_files(bmg_ctx* ctx)
{
  if (!ctx->opt.write_files || !ctx->files.empty()) return;
  ctx->files.resize(ctx->C);
  for (uint32_t c = 0; c < ctx->C; ++c) {
    ChainFiles& f = ctx->files[c];
    std::string b = std::string(ctx->opt.basename) + std::to_string(c);
    auto ob = [&](std::ofstream& s, const char* suf, bool bin) {
      s.open((b + suf).c_str(), bin ? std::ios::binary : std::ios::out);
      if (!s.is_open()) throw bmg_error(BMG_EIO, "Failed to open file: " + b + suf);
    };
    ob(f.log, "_log.txt", false);
    f.log << std::setprecision(3) << std::fixed;
    ob(f.loci, "_loci.dat", true);
    ob(f.modelsize, "_modelsize.dat", true);
    ob(f.jumpdistance, "_jumpdistance.dat", true);
    ob(f.log_likelihood, "_log_likelihood.dat", true);
    ob(f.log_prior, "_log_prior.dat", true);
    ob(f.move_type, "_move_type.dat", true);
    ob(f.move_size, "_move_size.dat", true);
    ob(f.pve, "_pve.dat", true);
    ob(f.alpha, "_alpha.dat", true);
    ob(f.sigma2, "_sigma2.dat", true);
    if (ctx->opt.n_types > 1) ob(f.types, "_types.dat", true);
    if (ctx->opt.save_beta) ob(f.beta, "_beta.dat", true);
    f.log << "output " << b << std::endl
          << "seed " << ctx->seeds[c] << std::endl
          << "type (PMV = 0, NK = 1, KSC = 2, G = 3) " << 0 << std::endl
          << "----------------------------------------------------" << std::endl;
    f.open = true;
  }
}

template <class T>
static void d2h(bmg_ctx* ctx, std::vector<T>& h, const T* d, size_t count)
{
  h.resize(count);
  if (count) CK(cudaMemcpyAsync(h.data(), d, sizeof(T) * count, cudaMemcpyDeviceToHost, ctx->stream));
}

static void drain_traces(bmg_ctx* ctx, uint64_t iter0, const bmg_trace_sink* sink)
{
  const DevTrace& tr = ctx->K.tr;
  const uint32_t C = ctx->C;
  d2h(ctx, ctx->h_jump, tr.jump, (size_t)C * tr.iter_cap);
  d2h(ctx, ctx->h_mtype, tr.mtype, (size_t)C * tr.iter_cap);
  d2h(ctx, ctx->h_msize, tr.msize, (size_t)C * tr.iter_cap);
  d2h(ctx, ctx->h_msz, tr.msz, (size_t)C * tr.thin_cap);
  d2h(ctx, ctx->h_ll, tr.ll, (size_t)C * tr.thin_cap);
  d2h(ctx, ctx->h_lp, tr.lp, (size_t)C * tr.thin_cap);
  d2h(ctx, ctx->h_s2, tr.s2, (size_t)C * tr.thin_cap);
  d2h(ctx, ctx->h_alpha, tr.alpha, (size_t)C * tr.thin_cap);
  d2h(ctx, ctx->h_pve, tr.pve, (size_t)C * tr.thin_cap * 3);
  d2h(ctx, ctx->h_log, tr.logrec, (size_t)C * tr.log_cap * BMG_LOGREC);
  CK(cudaMemcpyAsync(ctx->ch_h.data(), ctx->K.ch, sizeof(DevChain) * C, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  // loci / types / beta: only the used prefix of each chain
  ctx->h_loci.resize((size_t)C * tr.loci_cap);
  ctx->h_types.resize((size_t)C * tr.loci_cap);
  ctx->h_beta.resize((size_t)C * tr.beta_cap);
  for (uint32_t c = 0; c < C; ++c) {
    const DevChain& h = ctx->ch_h[c];
    if (h.tr_loci) {
      CK(cudaMemcpyAsync(&ctx->h_loci[(size_t)c * tr.loci_cap], tr.loci + (size_t)c * tr.loci_cap,
                         4 * (size_t)h.tr_loci, cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaMemcpyAsync(&ctx->h_types[(size_t)c * tr.loci_cap], tr.types + (size_t)c * tr.loci_cap,
                         (size_t)h.tr_loci, cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (h.tr_beta)
      CK(cudaMemcpyAsync(&ctx->h_beta[(size_t)c * tr.beta_cap], tr.beta + (size_t)c * tr.beta_cap,
                         8 * (size_t)h.tr_beta, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  for (uint32_t c = 0; c < C; ++c) {
    const DevChain& h = ctx->ch_h[c];
    bmg_trace_chunk k;
    std::memset(&k, 0, sizeof(k));
    k.chain = c;
    k.iter0 = iter0;
    k.n_iter = h.tr_iter;
    k.jumpdistance = &ctx->h_jump[(size_t)c * tr.iter_cap];
    k.move_type = &ctx->h_mtype[(size_t)c * tr.iter_cap];
    k.move_size = &ctx->h_msize[(size_t)c * tr.iter_cap];
    k.n_thin = h.tr_thin;
    k.modelsize = &ctx->h_msz[(size_t)c * tr.thin_cap];
    k.n_loci = h.tr_loci;
    k.loci = &ctx->h_loci[(size_t)c * tr.loci_cap];
    k.types = ctx->opt.n_types > 1 ? &ctx->h_types[(size_t)c * tr.loci_cap] : nullptr;
    k.log_likelihood = &ctx->h_ll[(size_t)c * tr.thin_cap];
    k.log_prior = &ctx->h_lp[(size_t)c * tr.thin_cap];
    k.sigma2 = &ctx->h_s2[(size_t)c * tr.thin_cap];
    k.alpha = &ctx->h_alpha[(size_t)c * tr.thin_cap];
    k.pve = &ctx->h_pve[(size_t)c * tr.thin_cap * 3];
    k.n_beta = h.tr_beta;
    k.beta = ctx->opt.save_beta ? &ctx->h_beta[(size_t)c * tr.beta_cap] : nullptr;
    if (sink && sink->fn) sink->fn(sink->user, &k);
    if (ctx->opt.write_files) {
      ChainFiles& f = ctx->files[c];
      f.jumpdistance.write((const char*)k.jumpdistance, k.n_iter);
      f.move_type.write((const char*)k.move_type, k.n_iter);
      f.move_size.write((const char*)k.move_size, k.n_iter);
      size_t lo = 0;
      for (uint64_t t = 0; t < k.n_thin; ++t) {
        uint32_t ms = k.modelsize[t];
        f.modelsize.write((const char*)&k.modelsize[t], 4);
        f.loci.write((const char*)&k.loci[lo], 4 * (size_t)ms);
        if (ctx->opt.n_types > 1) f.types.write((const char*)&k.types[lo], ms);
        lo += ms;
        f.log_likelihood.write((const char*)&k.log_likelihood[t], 8);
        f.log_prior.write((const char*)&k.log_prior[t], 8);
        f.sigma2.write((const char*)&k.sigma2[t], 8);
        f.pve.write((const char*)&k.pve[3 * t], 24);
        f.alpha.write((const char*)&k.alpha[t], 8);
      }
      if (ctx->opt.save_beta && k.n_beta) f.beta.write((const char*)k.beta, 8 * k.n_beta);
      // _log.txt lines (src/sampler.cpp:813-833)
      for (uint32_t g = 0; g < h.tr_log; ++g) {
        const double* r = &ctx->h_log[((size_t)c * tr.log_cap + g) * BMG_LOGREC];
        f.log << "(" << (uint64_t)r[0] << ")"
              << " acc.rate " << r[1] / r[0] << " acc.rate2 " << r[2] / r[3] << " acc.rate3 " << r[4] / r[5]
              << " p_move_size " << r[6] << " model size " << (uint64_t)r[7] << " log p " << r[8] << " PVE "
              << r[9] << "/" << r[10] << "/" << r[11] << " sigma2 " << r[12] << std::endl;
      }
      f.log.flush();
    }
  }
}

// learned: the RB step with this index (from 0) refreshes the MLP part when
// the proposal still adapts and the index is a multiple of `every`
static std::vector<Segment> plan_chunk(uint64_t first_iter, uint64_t chunk, uint64_t n_rao, uint64_t rb0,
                                       bool learned, uint64_t adapt_rb, bool always, uint64_t every)
{
  std::vector<Segment> segs;
  uint64_t t = first_iter, i = 0, rb = rb0;
  while (i < chunk) {
    const uint64_t next_rb = ((t / n_rao) + 1) * n_rao - 1;  // first iter >= t with (iter+1) % n_rao == 0
    const uint64_t seg = std::min<uint64_t>(chunk - i, next_rb - t + 1);
    t += seg;
    i += seg;
    const bool is_rb = t - 1 == next_rb;
    // the adaptive proposal's last adaptation is RB step adapt_rb - 2
    // (src/sampler.cpp:739-760); the MLP part follows the same rule
    const bool refresh = learned && is_rb && (always || rb + 1 < adapt_rb) && rb % every == 0;
    segs.push_back({seg, is_rb, refresh});
    if (is_rb) ++rb;
  }
  return segs;
}

// Issue a chunk on the context stream, with an event before the move kernel,
// after it, after the scan and after the rebuild of every segment.
static void issue_chunk(bmg_ctx* ctx, const std::vector<Segment>& segs)
{
  const DevConst& K = ctx->K;
  bmg_trace_reset_kernel<<<(ctx->C + 127) / 128, 128, 0, ctx->stream>>>(K.ch, (int)ctx->C);
  LAUNCHED(ctx, "bmg_trace_reset_kernel");
  const unsigned rec = ctx->capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
  for (size_t q = 0; q < segs.size(); ++q) {
    cudaEvent_t* ev = &ctx->seg_ev[4 * q];
    CK(cudaEventRecordWithFlags(ev[0], ctx->stream, rec));
    bmg_move_kernel<<<ctx->C, BMG_MOVE_THREADS, ctx->move_smem, ctx->stream>>>(K, (int)segs[q].iters);
    LAUNCHED(ctx, "bmg_move_kernel");
    CK(cudaEventRecordWithFlags(ev[1], ctx->stream, rec));
    if (segs[q].rb) {
      launch_scan(ctx);
      CK(cudaEventRecordWithFlags(ev[2], ctx->stream, rec));
      launch_rebuild(ctx, 0);
      if (segs[q].refresh) {
        CK(bmg_mlp_refresh(&K, ctx->km, (int)ctx->opt.learned_steps, (float)ctx->opt.learned_lr, ctx->adam_t,
                           ctx->stream));
        // LD feature, per step training + Adam + counter, forward pass, tables
        const uint64_t n = 4 + 3ull * ctx->opt.learned_steps;
        if (ctx->capturing) ctx->graph_launches += n;
        else ctx->n_launches += n;
        if (ctx->sync_check) CK(cudaStreamSynchronize(ctx->stream));
      }
      CK(cudaEventRecordWithFlags(ev[3], ctx->stream, rec));
    }
  }
}

extern "C" bmg_status bmg_run(bmg_ctx* ctx, uint64_t n_iter, const bmg_trace_sink* sink)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  if (ctx->n_iter == 0) ctx->t_start = time(nullptr);
  open_files(ctx);
  const uint64_t n_rao = ctx->opt.n_rao;
  const uint32_t gi = ctx->opt.graph_iters ? ctx->opt.graph_iters : 64;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, ctx->stream));
  uint64_t done = 0;
  while (done < n_iter) {
    const uint64_t chunk = std::min<uint64_t>(n_iter - done, gi);
    const uint64_t iter0 = ctx->n_iter;
    const std::vector<Segment> segs =
        plan_chunk(iter0, chunk, n_rao, ctx->rb_steps, ctx->K.lrn.on != 0, ctx->opt.n_rao_burnin,
                   ctx->opt.adaptation != 0, ctx->opt.learned_every ? ctx->opt.learned_every : 1);
    while (ctx->seg_ev.size() < 4 * segs.size()) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      ctx->seg_ev.push_back(e);
    }
    // a graph once the scan's launch shape is settled (its tuner reads
    // timings between launches); BMG_EAGER=1 or BMG_SYNC_CHECK=1 keep plain
    // launches
    const bool tuning = ctx->opt.scan_impl == BMG_SCAN_TCGEN05 && ctx->tc_forced < 0 && ctx->tc_variant < 0;
    const bool graph = !ctx->eager && !ctx->sync_check && !tuning;
    if (graph) {
      if (!ctx->graph_exec || !(ctx->graph_segs == segs)) {
        if (ctx->graph_exec) {
          cudaGraphExecDestroy(ctx->graph_exec);
          ctx->graph_exec = nullptr;
        }
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        ctx->capturing = true;
        ctx->graph_launches = 0;
        try {
          issue_chunk(ctx, segs);
        } catch (...) {
          ctx->capturing = false;
          cudaStreamEndCapture(ctx->stream, &g);
          if (g) cudaGraphDestroy(g);
          throw;
        }
        ctx->capturing = false;
        CK(cudaStreamEndCapture(ctx->stream, &g));
        cudaError_t ie = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
        cudaGraphDestroy(g);
        CK(ie);
        ctx->graph_segs = segs;
      }
      CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
      ctx->n_launches += ctx->graph_launches;
    } else {
      issue_chunk(ctx, segs);
    }
    CK(cudaStreamSynchronize(ctx->stream));
    for (size_t q = 0; q < segs.size(); ++q) {
      cudaEvent_t* ev = &ctx->seg_ev[4 * q];
      float a = 0, b = 0, c2 = 0;
      CK(cudaEventElapsedTime(&a, ev[0], ev[1]));
      ctx->ms[0] += a;
      if (segs[q].rb) {
        CK(cudaEventElapsedTime(&b, ev[1], ev[2]));
        CK(cudaEventElapsedTime(&c2, ev[2], ev[3]));
        ctx->ms[1] += b;
        ctx->ms[2] += c2;
        ctx->n_scans++;
      }
      ctx->n_iter += segs[q].iters;
      if (segs[q].rb) ++ctx->rb_steps;
    }
    drain_traces(ctx, iter0, sink);
    device_error_check(ctx);
    done += chunk;
  }
  CK(cudaEventRecord(e1, ctx->stream));
  CK(cudaEventSynchronize(e1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  ctx->ms[3] += ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_scan(bmg_ctx* ctx, double* p_r, double* p_r_types)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  DevConst& K = ctx->K;
  bmg_rbprep_kernel<<<ctx->C, BMG_MOVE_THREADS, ctx->move_smem, ctx->stream>>>(K, 0, 0.0);
  LAUNCHED(ctx, "bmg_rbprep_kernel");
  launch_scan(ctx);
  const size_t pc = (size_t)ctx->p * ctx->C;
  if (p_r) CK(cudaMemcpyAsync(p_r, K.p_r, 8 * pc, cudaMemcpyDeviceToHost, ctx->stream));
  if (p_r_types && ctx->opt.n_types > 1)
    CK(cudaMemcpyAsync(p_r_types, K.p_r_types, 8 * pc * ctx->opt.n_types, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  device_error_check(ctx);
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_scan_yhat(bmg_ctx* ctx, const double* y_hat, double sigma2, double* p_r,
                                    double* logodds)
{
  if (!ctx || !y_hat) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  if (!(sigma2 > 0) || !std::isfinite(sigma2)) throw bmg_error(BMG_EINVAL, "sigma2 must be positive and finite");
  DevConst& K = ctx->K;
  const size_t pc = (size_t)ctx->p * ctx->C;
  double amax = 0;
  for (uint64_t i = 0; i < ctx->n; ++i) {
    if (!std::isfinite(y_hat[i])) throw bmg_error(BMG_EINVAL, "y_hat must be finite");
    amax = std::max(amax, std::fabs(y_hat[i]));
  }
  if (!ctx->yhat_given) ctx->yhat_given = ctx->dalloc<double>((size_t)ctx->n * ctx->C, false);
  for (uint32_t c = 0; c < ctx->C; ++c)
    CK(cudaMemcpyAsync(ctx->yhat_given + (size_t)c * ctx->n, y_hat, 8 * ctx->n, cudaMemcpyHostToDevice,
                       ctx->stream));
  if (logodds && !ctx->lml_buf) ctx->lml_buf = ctx->dalloc<double>(pc, false);
  bmg_set_sigma2_kernel<<<(ctx->C + 127) / 128, 128, 0, ctx->stream>>>(K, sigma2);
  LAUNCHED(ctx, "bmg_set_sigma2_kernel");
  DevConst Ky = K;
  Ky.yhat = ctx->yhat_given;
  bmg_rbprep_kernel<<<ctx->C, BMG_MOVE_THREADS, ctx->move_smem, ctx->stream>>>(Ky, 1, amax);
  LAUNCHED(ctx, "bmg_rbprep_kernel");
  double* const before = K.p_lml;
  if (logodds) K.p_lml = ctx->lml_buf;
  try {
    launch_scan(ctx);
  } catch (...) {
    K.p_lml = before;
    throw;
  }
  K.p_lml = before;
  if (p_r) CK(cudaMemcpyAsync(p_r, K.p_r, 8 * pc, cudaMemcpyDeviceToHost, ctx->stream));
  if (logodds) CK(cudaMemcpyAsync(logodds, ctx->lml_buf, 8 * pc, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  device_error_check(ctx);
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_scan_logodds(bmg_ctx* ctx, double* logodds)
{
  if (!ctx || !logodds) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  DevConst& K = ctx->K;
  const size_t pc = (size_t)ctx->p * ctx->C;
  if (!ctx->lml_buf) ctx->lml_buf = ctx->dalloc<double>(pc, false);
  double* const before = K.p_lml;
  K.p_lml = ctx->lml_buf;
  try {
    bmg_rbprep_kernel<<<ctx->C, BMG_MOVE_THREADS, ctx->move_smem, ctx->stream>>>(K, 0, 0.0);
    LAUNCHED(ctx, "bmg_rbprep_kernel");
    launch_scan(ctx);
  } catch (...) {
    K.p_lml = before;
    throw;
  }
  K.p_lml = before;
  CK(cudaMemcpyAsync(logodds, ctx->lml_buf, 8 * pc, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  device_error_check(ctx);
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_scan_schur(bmg_ctx* ctx, double* dlml)
{
  if (!ctx || !dlml) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  if (ctx->multi) throw bmg_error(BMG_EUNSUPPORTED, "the Schur scan needs one phenotype per context");
  if (ctx->K.miss_total) throw bmg_error(BMG_EUNSUPPORTED, "the Schur scan does not take missing genotype calls");
  const uint32_t C = ctx->C;
  const size_t out_n = (size_t)C * ctx->p * ctx->K.n_terms;
  if (!ctx->schur_out) ctx->schur_out = ctx->dalloc<double>(out_n, false);
  std::vector<DevModel> mods(C);
  CK(cudaMemcpyAsync(mods.data(), ctx->K.cur, sizeof(DevModel) * C, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  std::vector<int> xcols(C);
  for (uint32_t c = 0; c < C; ++c) xcols[c] = mods[c].xcols;
  const int rc = bmg_schur_launch(&ctx->K, xcols.data(), &ctx->schur_bm, &ctx->schur_bm_cap, ctx->schur_out,
                                  ctx->stream);
  if (rc == 100) throw bmg_error(BMG_EUNSUPPORTED, "the Schur scan supports models of at most 128 columns");
  if (rc != 0)
    throw bmg_error(BMG_ECUDA, "Schur scan launch failed (step " + std::to_string(rc) +
                                   "): " + cudaGetErrorString(cudaGetLastError()));
  LAUNCHED(ctx, "bmg_schur_tc_kernel");
  CK(cudaMemcpyAsync(dlml, ctx->schur_out, 8 * out_n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  device_error_check(ctx);
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_learned_snapshot(bmg_ctx* ctx, float* theta, float* logit, float* features,
                                           uint32_t* t_snp, double* t_s, uint32_t* t_n)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  const DevLearned& L = ctx->K.lrn;
  if (!L.on) throw bmg_error(BMG_EINVAL, "the learned proposal is not on");
  const size_t pc = (size_t)ctx->p * ctx->C;
  // logits of the current parameters at the current state (the candidate
  // tables are left as the last refresh made them)
  if (logit) CK(bmg_mlp_forward(&ctx->K, ctx->stream));
  if (theta) CK(cudaMemcpyAsync(theta, L.theta, sizeof(float) * MLP_NPAR, cudaMemcpyDeviceToHost, ctx->stream));
  if (logit) CK(cudaMemcpyAsync(logit, L.logit, sizeof(float) * pc, cudaMemcpyDeviceToHost, ctx->stream));
  if (t_snp) CK(cudaMemcpyAsync(t_snp, L.t_snp, 4 * (size_t)ctx->C * L.topk, cudaMemcpyDeviceToHost, ctx->stream));
  if (t_s) CK(cudaMemcpyAsync(t_s, L.t_s, 8 * (size_t)ctx->C * L.topk, cudaMemcpyDeviceToHost, ctx->stream));
  if (t_n) CK(cudaMemcpyAsync(t_n, L.t_n, 4 * (size_t)ctx->C, cudaMemcpyDeviceToHost, ctx->stream));
  if (features) {
    float* d = nullptr;
    CK(cudaMallocAsync(&d, sizeof(float) * pc * MLP_F, ctx->stream));
    cudaError_t e = bmg_mlp_features(&ctx->K, d, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(features, d, sizeof(float) * pc * MLP_F, cudaMemcpyDeviceToHost, ctx->stream);
    cudaFreeAsync(d, ctx->stream);
    CK(e);
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_learned_grad(bmg_ctx* ctx, const uint32_t* rows, uint32_t n_rows, float* grad)
{
  if (!ctx || !rows || !grad || n_rows == 0) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  if (!ctx->K.lrn.on) throw bmg_error(BMG_EINVAL, "the learned proposal is not on");
  uint32_t* d = nullptr;
  CK(cudaMallocAsync(&d, 8 * (size_t)n_rows, ctx->stream));
  cudaError_t e = cudaMemcpyAsync(d, rows, 8 * (size_t)n_rows, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = bmg_mlp_grad(&ctx->K, ctx->adam_t, d, n_rows, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(grad, ctx->K.lrn.grad, sizeof(float) * MLP_NPAR, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->K.lrn.grad, 0, sizeof(float) * MLP_NPAR, ctx->stream);
  cudaFreeAsync(d, ctx->stream);
  CK(e);
  CK(cudaStreamSynchronize(ctx->stream));
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_get_state(bmg_ctx* ctx, uint32_t chain, bmg_chain_state* st, uint32_t* loci,
                                    uint8_t* type_inds, uint32_t loci_cap)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  if (chain >= ctx->C || !st) throw bmg_error(BMG_EINVAL, "chain index");
  DevModel M;
  DevChain h;
  CK(cudaMemcpyAsync(&M, ctx->K.cur + chain, sizeof(M), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(&h, ctx->K.ch + chain, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  std::vector<uint32_t> lc(M.k);
  std::vector<uint8_t> ti(M.k);
  if (M.k) {
    CK(cudaMemcpyAsync(lc.data(), M.loci, 4 * (size_t)M.k, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(ti.data(), M.type_inds, (size_t)M.k, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  st->model_size = (uint32_t)M.k;
  st->log_likelihood = M.ll;
  // log prior from the same tables the device uses
  {
    double lp = 0;
    int ng = 0;
    const uint32_t tw = ctx->K.tw;
    std::vector<double> tab((size_t)22 * tw);
    CK(cudaMemcpyAsync(tab.data(), ctx->K.tab, 8 * tab.size(), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < 5; ++i)
      if (ctx->K.allow_types[i]) { lp += tab[(size_t)(14 + i) * tw + M.Ns[i]]; ng += M.Ns[i]; }
    lp += tab[(size_t)19 * tw + ng] + tab[(size_t)20 * tw + ng] - tab[(size_t)21 * tw + ng];
    st->log_prior = lp;
  }
  st->sigma2 = M.sigma2;
  st->alpha = h.alpha;
  st->n_iter = h.n_iter;
  st->n_accepted = h.n_accepted;
  st->p_move_size = h.p_move_size;
  st->rng_draws = h.rng.slot;
  for (int i = 0; i < M.k && (uint32_t)i < loci_cap; ++i) {
    if (loci) loci[i] = lc[i];
    if (type_inds) type_inds[i] = ti[i];
  }
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_get_rao(bmg_ctx* ctx, uint32_t chain, double* p_rao, double* p_rao_types)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  if (chain >= ctx->C) throw bmg_error(BMG_EINVAL, "chain index");
  const size_t p = ctx->p, nt = ctx->opt.n_types > 1 ? ctx->opt.n_types : 0;
  // DMA into pinned staging, then into the caller's memory
  ctx->ensure_stage(8 * p * std::max<size_t>(1, nt));
  CK(cudaEventSynchronize(ctx->stage_ev[0]));
  double* st = reinterpret_cast<double*>(ctx->stage[0]);
  if (p_rao) {
    CK(cudaMemcpyAsync(st, ctx->K.p_rao + chain * p, 8 * p, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    std::memcpy(p_rao, st, 8 * p);
  }
  if (p_rao_types && nt) {
    CK(cudaMemcpyAsync(st, ctx->K.p_rao_types + chain * p * nt, 8 * p * nt, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    std::memcpy(p_rao_types, st, 8 * p * nt);
  }
  return BMG_OK;
  API_END
}

// Device -> caller's memory through the two pinned staging buffers: the DMA
// of chunk i overlaps the host copy (several threads) of chunk i - 1.
static void copy_out_staged(bmg_ctx* ctx, const uint8_t* src, uint8_t* dst, size_t bytes)
{
  const size_t chunk = std::min<size_t>(bytes, size_t(32) << 20);
  ctx->ensure_stage(chunk);
  const unsigned nth = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
  auto host_copy = [&](const uint8_t* s, uint8_t* d, size_t n) {
    std::vector<std::thread> th;
    const size_t part = (n + nth - 1) / nth;
    for (unsigned t = 0; t < nth && t * part < n; ++t)
      th.emplace_back([=] { std::memcpy(d + t * part, s + t * part, std::min(part, n - t * part)); });
    for (auto& x : th) x.join();
  };
  size_t prev_off = 0, prev_n = 0;
  int b = 0, prev_b = -1;
  for (size_t off = 0; off < bytes; off += chunk, b ^= 1) {
    const size_t n = std::min(chunk, bytes - off);
    CK(cudaEventSynchronize(ctx->stage_ev[b]));
    CK(cudaMemcpyAsync(ctx->stage[b], src + off, n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaEventRecord(ctx->stage_ev[b], ctx->stream));
    if (prev_b >= 0) {
      CK(cudaEventSynchronize(ctx->stage_ev[prev_b]));
      host_copy(ctx->stage[prev_b], dst + prev_off, prev_n);
    }
    prev_b = b;
    prev_off = off;
    prev_n = n;
  }
  if (prev_b >= 0) {
    CK(cudaEventSynchronize(ctx->stage_ev[prev_b]));
    host_copy(ctx->stage[prev_b], dst + prev_off, prev_n);
  }
}

extern "C" bmg_status bmg_get_rao_all(bmg_ctx* ctx, double* p_rao, double* p_rao_types)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  const size_t p = ctx->p, C = ctx->C, nt = ctx->opt.n_types > 1 ? ctx->opt.n_types : 0;
  if (p_rao)
    copy_out_staged(ctx, reinterpret_cast<const uint8_t*>(ctx->K.p_rao), reinterpret_cast<uint8_t*>(p_rao),
                    8 * p * C);
  if (p_rao_types && nt)
    copy_out_staged(ctx, reinterpret_cast<const uint8_t*>(ctx->K.p_rao_types),
                    reinterpret_cast<uint8_t*>(p_rao_types), 8 * p * nt * C);
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_get_proposal(bmg_ctx* ctx, uint32_t chain, double* p_prop, double* p_prop_types)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  if (chain >= ctx->C) throw bmg_error(BMG_EINVAL, "chain index");
  const size_t p = ctx->p;
  if (p_prop) {
    // stored in the proposal tree's in-order position order
    std::vector<double> byq(p);
    std::vector<int32_t> pos, inv;
    inorder_ranks(p, pos, inv);
    CK(cudaMemcpyAsync(byq.data(), ctx->K.p_prop + chain * p, 8 * p, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (size_t j = 0; j < p; ++j) p_prop[j] = byq[pos[j]];
  }
  if (p_prop_types && ctx->opt.n_types > 1)
    CK(cudaMemcpyAsync(p_prop_types, ctx->K.p_prop_types + chain * p * ctx->opt.n_types,
                       8 * p * ctx->opt.n_types, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_get_last_scan(bmg_ctx* ctx, uint32_t chain, double* p_r, double* p_r_types)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  if (chain >= ctx->C) throw bmg_error(BMG_EINVAL, "chain index");
  const size_t p = ctx->p;
  if (p_r) CK(cudaMemcpyAsync(p_r, ctx->K.p_r + chain * p, 8 * p, cudaMemcpyDeviceToHost, ctx->stream));
  if (p_r_types && ctx->opt.n_types > 1)
    CK(cudaMemcpyAsync(p_r_types, ctx->K.p_r_types + chain * p * ctx->opt.n_types, 8 * p * ctx->opt.n_types,
                       cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return BMG_OK;
  API_END
}

extern "C" bmg_status bmg_get_timings(bmg_ctx* ctx, double* ms4)
{
  if (!ctx || !ms4) return BMG_EINVAL;
  for (int i = 0; i < 4; ++i) ms4[i] = ctx->ms[i];
  return BMG_OK;
}

extern "C" bmg_status bmg_reset_timings(bmg_ctx* ctx, uint64_t* n_scans)
{
  if (!ctx) return BMG_EINVAL;
  if (n_scans) *n_scans = ctx->n_scans;
  for (int i = 0; i < 4; ++i) ctx->ms[i] = 0;
  ctx->n_scans = 0;
  ctx->n_launches = 0;
  return BMG_OK;
}

extern "C" bmg_status bmg_get_scan_shape(bmg_ctx* ctx, int32_t* variant, char* name, size_t name_len)
{
  if (!ctx) return BMG_EINVAL;
  const int v = ctx->tc_forced >= 0 ? ctx->tc_forced : ctx->tc_variant;
  if (variant) *variant = v;
  if (name && name_len) {
    if (v >= 0) bmg_scan_tc_variant_name(v, name, name_len);
    else snprintf(name, name_len, "tuning");
  }
  return BMG_OK;
}

extern "C" __global__ void bmg_exp_selftest_kernel(const double* a, double* out, uint64_t n);

extern "C" bmg_status bmg_selftest_exp(const double* a, double* out, size_t n)
{
  if ((!a || !out) && n) return BMG_EINVAL;
  for (size_t i = 0; i < n; ++i)
    if (!(fabs(a[i]) <= 700.0)) return BMG_EINVAL;
  if (!n) return BMG_OK;
  double* d = nullptr;
  if (cudaMalloc(&d, 16 * n) != cudaSuccess) return BMG_ECUDA;
  bool ok = cudaMemcpy(d, a, 8 * n, cudaMemcpyHostToDevice) == cudaSuccess;
  if (ok) {
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 4096);
    bmg_exp_selftest_kernel<<<blocks, 256>>>(d, d + n, (uint64_t)n);
    ok = cudaGetLastError() == cudaSuccess && cudaMemcpy(out, d + n, 8 * n, cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  cudaFree(d);
  return ok ? BMG_OK : BMG_ECUDA;
}

extern "C" bmg_status bmg_get_scan_tuning(bmg_ctx* ctx, float* ms, int32_t n, int32_t* n_shapes)
{
  if (!ctx || (n > 0 && !ms)) return BMG_EINVAL;
  const int nv = bmg_scan_tc_variants();
  if (n_shapes) *n_shapes = nv;
  for (int i = 0; i < n && i < nv; ++i) ms[i] = i < (int)ctx->tc_ms.size() ? ctx->tc_ms[i] : -1.0f;
  return BMG_OK;
}

extern "C" bmg_status bmg_get_scan_shape_name(int32_t shape, char* name, size_t name_len)
{
  if (shape < 0 || shape >= bmg_scan_tc_variants() || !name || !name_len) return BMG_EINVAL;
  bmg_scan_tc_variant_name(shape, name, name_len);
  return BMG_OK;
}

extern "C" bmg_status bmg_get_launch_count(bmg_ctx* ctx, uint64_t* n_launches)
{
  if (!ctx || !n_launches) return BMG_EINVAL;
  *n_launches = ctx->n_launches;
  return BMG_OK;
}

extern "C" bmg_status bmg_finish(bmg_ctx* ctx)
{
  if (!ctx) return BMG_EINVAL;
  API_BEGIN
  check_ready(ctx);
  const bmg_options& o = ctx->opt;
  const uint32_t C = ctx->C;
  CK(cudaMemcpyAsync(ctx->ch_h.data(), ctx->K.ch, sizeof(DevChain) * C, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  double elapsed = ctx->t_start ? difftime(time(nullptr), ctx->t_start) : 0.0;
  for (uint32_t c = 0; c < C; ++c) {
    std::string b = std::string(o.basename) + std::to_string(c);
    const DevChain& h = ctx->ch_h[c];
    {  // src/samplerstats.hpp:92-110
      std::ofstream f((b + "_samplerstats.txt").c_str());
      if (!f.is_open()) throw bmg_error(BMG_EIO, "Failed to open file: " + b + "_samplerstats.txt");
      f << "n_likelihood_updates_on_add " << h.n_lik_add << std::endl
        << "n_likelihood_updates_on_rem " << h.n_lik_rem << std::endl
        << "n_likelihood_computations " << h.n_lik_full + 3 << std::endl
        << "sampling_time_in_seconds " << elapsed << std::endl
        << "mhmove_time_in_seconds " << ctx->ms[0] / 1000.0 << std::endl
        << "rao_time_in_seconds " << ctx->ms[1] / 1000.0 << std::endl
        << "clock_resolution_in_seconds " << 1e-9 << std::endl
        << "p_movesize " << h.p_move_size << std::endl;
    }
    if (!ctx->files.empty() && ctx->files[c].open) {
      ctx->files[c].log << "Elapsed time: " << elapsed << " seconds." << std::endl;
      ctx->files[c] = ChainFiles();
    }
    std::vector<double> rao(ctx->p), raot;
    if (o.n_types > 1) raot.resize(ctx->p * o.n_types);
    bmg_get_rao(ctx, c, rao.data(), o.n_types > 1 ? raot.data() : nullptr);
    std::ofstream fr((b + "_rao.dat").c_str(), std::ios::binary);
    if (!fr.is_open()) throw bmg_error(BMG_EIO, "Failed to open file: " + b + "_rao.dat");
    fr.write((const char*)rao.data(), 8 * rao.size());
    if (o.n_types > 1) {
      std::ofstream ft((b + "_rao_types.dat").c_str(), std::ios::binary);
      ft.write((const char*)raot.data(), 8 * raot.size());
    }
  }
  ctx->files.clear();
  {  // Prior::print (src/prior.hpp:221-243), basename of chain 0 without its index
    std::ofstream f((std::string(o.basename) + "_prior.txt").c_str());
    if (f.is_open()) {
      f << "a_omega = " << ctx->g_a << std::endl
        << "b_omega = " << ctx->g_b << std::endl
        << "nu_sigma2 = " << o.nu_sigma2 << std::endl
        << "s2_sigma2 = " << ctx->s2_sigma2 << std::endl
        << "mu_alpha = " << o.mu_alpha << std::endl;
      for (int t = 0; t < 5; ++t)
        f << "type_" << kTypeName[t] << " = " << ctx->K.types_prior[t] << " (allowed? " << ctx->K.allow_types[t]
          << ")" << std::endl;
      for (int t = 0; t < 4; ++t)
        f << "term_" << kTypeName[t] << " allowed = " << ctx->K.allow_terms[t] << std::endl
          << "nu_tau2_" << kTypeName[t] << " = " << ctx->K.nu_tau2[t] << std::endl
          << "s2_tau2_" << kTypeName[t] << " = " << ctx->K.s2_tau2[t] << std::endl;
    }
  }
  return BMG_OK;
  API_END
}

// data statistics the reference prints at start (src/main.cpp:58-62)
extern "C" bmg_status bmg_get_data_stats(bmg_ctx* ctx, double* out4)
{
  if (!ctx || !out4) return BMG_EINVAL;
  out4[0] = ctx->var_x;
  out4[1] = ctx->mean_x;
  out4[2] = ctx->var_y;
  out4[3] = ctx->yy;
  return BMG_OK;
}
