// The MCMC move kernel of libbmg: one CTA per chain.
//
// Warp 0 runs the reference's sampler control flow (src/sampler.cpp:551-834,
// src/sampler.hpp:899-1769) with every lane executing the scalar code, so the
// warp stays converged and all lanes hold the same values; lane-parallel
// loops do the O(k) and O(k^2) linear algebra.  All eight warps join for the
// n-wide phases (fitted values, PVE sums, alpha sufficient statistics, the
// fixed-point residual and its limbs for the scan).  Random numbers come from
// bmg_rng.h in the reference's draw order, so a chain reproduces the oracle's
// trajectory for the same seed.
//
// FP64 is used wherever the reference uses it on the move path: the Cholesky
// factor, its up/downdates (src/symmmatrix.cpp:144-195, src/dchex.f), the
// marginal likelihood and the MH ratio.  Genotype products are exact integers
// (popcounts on the 2-bit codes), and products with phenotypes or covariates
// use fixed-point integers.
#include <math.h>

#include "common.cuh"
#include "df64.h"
#include "flog.h"

#define TAB_ADD_A 0
#define TAB_REM_A 1
#define TAB_LT 2
#define TAB_LTM1 7
#define TAB_LS 12
#define TAB_LSM1 13
#define TAB_LGT 14
#define TAB_LGA 19
#define TAB_LGB 20
#define TAB_LGS 21

#define LOG_HALF_D -0.69314718055994528622676398299518041312694549560546875

// Cholesky factors and v of both models stay in shared memory while their
// order is at most SMK; larger models live in global memory (same packed
// upper-triangular layout: column c holds rows 0..c at c (c + 1) / 2).
#define SMK 128
#define SM_TRI (SMK * (SMK + 1) / 2)

struct MoveShared {
  DevModel mod[2];      // current (0) and proposed (1) model headers
  DevChain chs;         // the chain's dynamic state
  DevPheno phs;         // the chain's sample
  double Ls[2][SM_TRI];
  double vs[2][SMK];
  double tv[2][SMK];    // work vectors for beta and its mean
  double cs[SMK], sn[SMK];  // Givens rotations of a downdate
  int l_smem[2];        // factor and v of model i are in shared memory
  long long w_m;        // learned proposal: weight of the candidates outside the zero set (x 2^40)
  uint32_t move_inds[BMG_MAX_MS + 1];
  uint32_t move_add[BMG_MAX_MS + 1];
  uint32_t move_rem[BMG_MAX_MS + 1];
  long long move_map[BMG_MAX_MS + 1];
  uint8_t move_isadd[BMG_MAX_MS + 1];
  // dd_add flips relative to the prefix base
  int n_pend;
  int pend_snp[BMG_PEND_MAX];
  int pend_pos[BMG_PEND_MAX];
  long long pend_d[BMG_PEND_MAX];
  // dd_rem non-zero set, in in-order position order
  int n_rs;
  uint32_t rs_snp[BMG_REMSET_MAX];
  int rs_pos[BMG_REMSET_MAX];
  double rs_w[BMG_REMSET_MAX];
  uint8_t rs_on[BMG_REMSET_MAX];
  // bulk phase exchange
  long long bl[8][2];
  unsigned long long bi[8][4];  // per warp: 128-bit sums of the integer bulk phase (lo, hi pairs)
  double bd[8][6];
  double bsum[6];
  long long bsuml[2];
  double bmax[8];
  int bulk_mode;
  int bulk_s;           // fixed-point exponent of the bulk phase
  int bulk_nterm;       // genotype columns in the bulk phase
  int err;
  int iter_stop;        // stop after this iteration (RB step follows)
  int n_done;
  double bulk_b0;       // constant-term coefficient
  long long bulk_b0i;
  double bulk_e[BMG_MAX_COV + 1];  // covariate coefficients (the constant first)
  double yhat_given_max;  // max |y_hat| of a residual from given fitted values (BULK_YHAT)
  // n-wide products of warp 0's move, handed to all eight warps (help jobs)
  int job_kind;
  int job_r0, job_r1, job_term;
  uint32_t job_snp;
  const DevModel* job_M;
  double* job_out;
  long long job_part[BMG_MOVE_THREADS / 32];
  // delayed rejection: the exhaustive model's scalars and, per moved SNP
  // (bit order), its proposal weights
  int dr_ms, dr_vs, dr_llen, dr_Ns[5];
  double dr_syx, dr_ldq, dr_ldqx, dr_lmp;
  double dr_qa[BMG_DR_MAX], dr_qr[BMG_DR_MAX], dr_lqt[BMG_DR_MAX];
  int dr_b2o[BMG_DR_MAX];
};

// genotype columns of the bulk phase: snp, term, fixed-point coefficient
#define BULK_MAXCOL 1024
struct BulkCols {
  uint32_t snp[BULK_MAXCOL];
  int8_t term[BULK_MAXCOL];
  long long coef[BULK_MAXCOL];
};

// ------------------------------------------------------------------ helpers

#define HELP_BAR 1  // named barrier of warp 0 and its seven helper warps
enum { HJ_EXIT = 0, HJ_CROSS = 1, HJ_XY = 2 };

__device__ __forceinline__ void bar_sync_all()
{
  asm volatile("bar.sync %0, %1;" ::"r"(HELP_BAR), "r"(BMG_MOVE_THREADS) : "memory");
}

// Exact sum_i x_t(g_a,i) x_u(g_snp,i) between the new genotype column
// (snp, term) and the model's genotype columns r0 <= r < r1, four columns at
// a time: warp `wid` of `nwarps` takes the groups wid, wid + nwarps, ...; a
// word of the new column is loaded once per four model columns and the four
// rows' loads are independent.  Exact integer popcounts.
__device__ void cross_cols_part(const DevConst& K, const DevPheno& P, const DevModel* M, int r0, int r1,
                                uint32_t snp, int term, double* out, int wid, int nwarps)
{
  const int lane = threadIdx.x & 31;
  const uint64_t* rb = (const uint64_t*)(K.geno + (size_t)snp * K.gs);
  const unsigned nw64 = K.gs / 8;
  const uint64_t m5 = 0x5555555555555555ull;
  const int cHu = coefH(term), cRu = coefR(term);
  for (int r = r0 + 4 * wid; r < r1; r += 4 * nwarps) {
    const int cnt = min(4, r1 - r);
    const uint64_t* ra[4];
    int cH[4], cR[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = r + min(q, cnt - 1);
      ra[q] = (const uint64_t*)(K.geno + (size_t)M->xc_snp[idx] * K.gs);
      cH[q] = coefH(M->xc_type[idx]);
      cR[q] = coefR(M->xc_type[idx]);
    }
    int hh[4] = {0, 0, 0, 0}, hr[4] = {0, 0, 0, 0}, rh[4] = {0, 0, 0, 0}, rr[4] = {0, 0, 0, 0};
#pragma unroll 4
    for (unsigned w = lane; w < nw64; w += 32) {
      const uint64_t y = rb[w];
      const uint64_t yh = (y >> 1) & (P.mask2 ? P.mask2[w] : m5), yl = y & m5;
      const uint64_t Hy = yh & ~yl, Ry = yh & yl;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint64_t x = ra[q][w];
        const uint64_t xh = (x >> 1) & m5, xl = x & m5;
        const uint64_t Hx = xh & ~xl, Rx = xh & xl;
        hh[q] += __popcll(Hx & Hy);
        hr[q] += __popcll(Hx & Ry);
        rh[q] += __popcll(Rx & Hy);
        rr[q] += __popcll(Rx & Ry);
      }
    }
    long long v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
      v[q] = (long long)cH[q] * cHu * hh[q] + (long long)cH[q] * cRu * hr[q] +
             (long long)cR[q] * cHu * rh[q] + (long long)cR[q] * cRu * rr[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] += __shfl_xor_sync(FULL_MASK, v[q], o);
    }
    if (lane == 0)
      for (int q = 0; q < cnt; ++q) out[r + q] = (double)v[q];
  }
}

// sum_i x_term(g_snp,i) yint_i over the words of thread t of nth (the
// phenotype is zero outside the sample); the caller reduces
__device__ long long geno_dot_part(const DevConst& K, const DevPheno& P, uint32_t snp, int term, int t, int nth)
{
  const uint32_t* row = reinterpret_cast<const uint32_t*>(K.geno + (size_t)snp * K.gs);
  const long long cH = coefH(term), cR = coefR(term);
  long long acc = 0;
  for (uint32_t w = t; w < (uint32_t)(K.gs / 4); w += nth) {
    const uint32_t code = row[w];
    if (!code) continue;
    for (int q = 0; q < 16; ++q) {
      const uint32_t c2 = (code >> (2 * q)) & 3u;
      if (c2 >= 2u) acc += (c2 == 2u ? cH : cR) * P.yint[(size_t)16 * w + q];
    }
  }
  return acc;
}

// Warps 1-7 while warp 0 runs a move: wait for a job, do this warp's share,
// meet again; until warp 0 posts HJ_EXIT.
__device__ void help_loop(const DevConst& K, MoveShared& s)
{
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (;;) {
    bar_sync_all();
    const int kind = s.job_kind;
    if (kind == HJ_EXIT) break;
    if (kind == HJ_CROSS) {
      cross_cols_part(K, s.phs, s.job_M, s.job_r0, s.job_r1, s.job_snp, s.job_term, s.job_out, wid,
                      BMG_MOVE_THREADS / 32);
    } else if (kind == HJ_XY) {
      const long long a = warp_sum_ll(geno_dot_part(K, s.phs, s.job_snp, s.job_term, threadIdx.x, BMG_MOVE_THREADS));
      if (lane == 0) s.job_part[wid] = a;
    }
    bar_sync_all();
  }
}

struct Warp {
  const DevConst& K;
  const DevPheno& P;    // the chain's sample (shared-memory copy)
  int c;
  DevChain* ch;
  DevModel* cur;
  DevModel* nm;
  MoveShared& s;
  int lane;
  bmg_rng_t rng;
  unsigned km;
  bool helpers = false;  // warps 1-7 wait in help_loop for n-wide jobs

  __device__ Warp(const DevConst& k, int chain, MoveShared& sh)
  : K(k), P(sh.phs), c(chain), ch(&sh.chs), cur(&sh.mod[0]), nm(&sh.mod[1]), s(sh),
    lane(threadIdx.x & 31), km(k.km)
  {
    rng = sh.chs.rng;
  }

  __device__ void fail(int code)
  {
    if (lane == 0 && s.err == 0) s.err = code;
    __syncwarp();
  }

  __device__ double u01() { return bmg_uniform01(&rng); }
  __device__ double nrm() { return bmg_normal(&rng); }

  /* src/rand.hpp:61-78 */
  __device__ double sinvchi2(double s2)
  {
    for (int t = 0; t < 64; ++t) {
      double g = bmg_gamma(&rng, 0.5 * P.rng_nu);
      if (isnan(g)) { fail(BMG_DERR_RNG); return 1.0; }
      double val = P.rng_nu * s2 / (2.0 * g);
      if (val > 0 && isfinite(val)) return val;
    }
    fail(BMG_DERR_RNG);
    return 1.0;
  }
  /* src/rand.hpp:85-97 */
  __device__ double sinvchi2(double nu, double s2)
  {
    for (int t = 0; t < 64; ++t) {
      double g = bmg_gamma(&rng, 0.5 * nu);
      if (isnan(g)) { fail(BMG_DERR_RNG); return 1.0; }
      double val = nu * s2 / (2.0 * g);
      if (val > 0 && isfinite(val)) return val;
    }
    fail(BMG_DERR_RNG);
    return 1.0;
  }
  /* src/utils.cpp:46-57 */
  __device__ int sample_naive(const double* cumsum, int m)
  {
    double z = cumsum[m - 1];
    double r = u01() * z;
    for (int i = 0; i < m; ++i)
      if (r < cumsum[i]) return i;
    fail(BMG_DERR_NAN);
    return m - 1;
  }

  __device__ const double* tab(int which) const { return K.tab + (size_t)which * K.tw; }

  /* src/prior.hpp:144-167 from the host tables */
  __device__ double lchange_add(const int* Ns, int nl, int type) const
  {
    return tab(TAB_ADD_A)[nl] + (tab(TAB_LT + type)[Ns[type]] - tab(TAB_LS)[nl]);
  }
  __device__ double lchange_rem(const int* Ns, int nl, int type) const
  {
    return tab(TAB_REM_A)[nl] + (tab(TAB_LSM1)[nl] - tab(TAB_LTM1 + type)[Ns[type]]);
  }
  __device__ double lchange_swi(const int* Ns, int ta, int tr) const
  {
    return (ta == tr) ? 0 : tab(TAB_LT + ta)[Ns[ta]] - tab(TAB_LTM1 + tr)[Ns[tr]];
  }
  /* src/prior.hpp:169-183 */
  __device__ double log_model(const int* Ns) const
  {
    double lp = 0;
    int ng = 0;
    for (int i = 0; i < 5; ++i) {
      if (K.allow_types[i]) {
        lp += tab(TAB_LGT + i)[Ns[i]];
        ng += Ns[i];
      }
    }
    lp += tab(TAB_LGA)[ng] + tab(TAB_LGB)[ng] - tab(TAB_LGS)[ng];
    return lp;
  }
  __device__ double sample_inv_tau2_prior(int type)
  {
    if (K.use_individual_tau2) return 1.0 / (ch->alpha2 * sinvchi2(K.nu_tau2[type], K.s2_tau2[type]));
    return ch->inv_t2a2[type];
  }

  // dd_add weight of a SNP (fixed point) and as double
  __device__ long long qadd_int(uint32_t snp) const
  {
    double pp = K.p_prop[(size_t)c * K.p + K.pos[snp]];
    double w = fmax(pp, K.q_add_min);
    return __double2ll_rn(w * ldexp(1.0, K.qs));
  }
  __device__ double qadd(uint32_t snp) const { return (double)qadd_int(snp) * ldexp(1.0, -K.qs); }
  __device__ double qrem(uint32_t snp) const
  {
    double pp = K.p_prop[(size_t)c * K.p + K.pos[snp]];
    return fmax(1.0 - pp, K.q_rem_min);
  }
  // q_add_types and their cumulative sums (src/sampler.cpp:526-544)
  __device__ void qtypes(uint32_t snp, double* qa, double* qcum) const
  {
    const double* pt = K.p_prop_types + ((size_t)c * K.p + snp) * K.n_types;
    for (unsigned t = 0; t < K.n_types; ++t) {
      qa[t] = fmax(pt[t], K.q_add_min);
      qcum[t] = (t == 0) ? qa[t] : qcum[t - 1] + qa[t];
    }
  }

  // ------------------------------------------------------- model arrays
  __device__ static size_t TRI(int r, int col) { return (size_t)col * (col + 1) / 2 + r; }
  __device__ int midx(const DevModel* M) const { return M == cur ? 0 : 1; }
  __device__ double* Lb(const DevModel* M) const
  {
    int i = midx(M);
    return s.l_smem[i] ? s.Ls[i] : M->l;
  }
  __device__ double* Vb(const DevModel* M) const
  {
    int i = midx(M);
    return s.l_smem[i] ? s.vs[i] : M->v;
  }
  __device__ double& XX(DevModel* M, int r, int col) const { return M->xx[(size_t)col * km + r]; }
  __device__ double& L(DevModel* M, int r, int col) const { return Lb(M)[TRI(r, col)]; }

  // move a model's factor and v from shared to global memory (it outgrew SMK)
  __device__ void spill(DevModel* M)
  {
    int i = midx(M);
    if (!s.l_smem[i]) return;
    size_t tri = TRI(0, min(M->llen, SMK));
    for (size_t q = lane; q < tri; q += 32) M->l[q] = s.Ls[i][q];
    for (int q = lane; q < min(M->vlen, SMK); q += 32) M->v[q] = s.vs[i][q];
    __syncwarp();
    if (lane == 0) s.l_smem[i] = 0;
    __syncwarp();
  }

  /* src/model.hpp:115-162: copy the active parts of a model */
  __device__ void copy_model(DevModel* d, const DevModel* src)
  {
    int xc = src->xcols, ll = src->llen;
    if (ll > SMK || src->vlen > SMK) spill(d);
    for (int col = 0; col < xc; ++col)
      for (int r = lane; r <= col; r += 32) d->xx[(size_t)col * km + r] = src->xx[(size_t)col * km + r];
    {
      const double* ls = Lb(src);
      double* ld = Lb(d);
      size_t tri = TRI(0, ll);
      for (size_t q = lane; q < tri; q += 32) ld[q] = ls[q];
    }
    for (int i = lane; i < xc; i += 32) {
      d->xy[i] = src->xy[i];
      d->inv[i] = src->inv[i];
      d->xc_snp[i] = src->xc_snp[i];
      d->xc_type[i] = src->xc_type[i];
    }
    {
      const double* vs = Vb(src);
      double* vd = Vb(d);
      for (int i = lane; i < src->vlen; i += 32) vd[i] = vs[i];
    }
    int vb = max(src->vlen, src->blen);
    for (int i = lane; i < vb; i += 32) {
      d->beta[i] = src->beta[i];
      d->mu_beta[i] = src->mu_beta[i];
    }
    for (int i = lane; i < src->k; i += 32) {
      d->loci[i] = src->loci[i];
      d->type_inds[i] = src->type_inds[i];
      d->x_ind1[i] = src->x_ind1[i];
      d->x_ind2[i] = src->x_ind2[i];
    }
    if (lane == 0) {
      d->k = src->k;
      d->xcols = src->xcols;
      d->llen = src->llen;
      d->vlen = src->vlen;
      d->blen = src->blen;
      for (int i = 0; i < 5; ++i) d->Ns[i] = src->Ns[i];
      d->mu_beta_computed = src->mu_beta_computed;
      d->sigma2 = src->sigma2;
      d->syx = src->syx;
      d->ldq = src->ldq;
      d->ldqx = src->ldqx;
      d->ll = src->ll;
    }
    __syncwarp();
  }

  // ------------------------------------------------------- linear algebra
  // An FP64 instruction occupies a GB300 SM sub-partition's FP64 pipe for
  // about 64 cycles whatever the number of active lanes (a dependent DFMA
  // takes 31 ns, a division 0.2 us, a log 1 us), so the solves below keep the
  // solution in registers, one element per lane and chunk of 32, and work
  // column by column: a step is one multiplication by the reciprocal of the
  // diagonal (all reciprocals taken up front, lane-parallel), a broadcast and
  // one FMA per chunk.  Orders beyond REG_N keep the memory-resident loops.
  static constexpr int REG_Q = 4;
  static constexpr int REG_N = 32 * REG_Q;

  // solve U' x = b in place (forward substitution), U = first len of L
  __device__ void trsv_T(const DevModel* M, double* x, int len)
  {
    const double* lb = Lb(M);
    if (len > REG_N) {
      for (int j = 0; j < len; ++j) {
        const double* colj = lb + TRI(0, j);
        double part = 0.0;
        for (int i = lane; i < j; i += 32) part += colj[i] * x[i];
        part = warp_sum_d(part);
        double xj = (x[j] - part) / colj[j];
        __syncwarp();
        if (lane == 0) x[j] = xj;
        __syncwarp();
      }
      return;
    }
    double xr[REG_Q], rd[REG_Q];
#pragma unroll
    for (int q = 0; q < REG_Q; ++q) {
      const int i = lane + 32 * q;
      xr[q] = (i < len) ? x[i] : 0.0;
      rd[q] = 0.0;
      if (32 * q < len) rd[q] = 1.0 / ((i < len) ? lb[TRI(i, i)] : 1.0);
    }
#pragma unroll
    for (int qc = 0; qc < REG_Q; ++qc) {
      if (32 * qc >= len) break;
      const int jend = min(32, len - 32 * qc);
      for (int jj = 0; jj < jend; ++jj) {
        const int j = 32 * qc + jj;
        const double xj = __shfl_sync(FULL_MASK, xr[qc] * rd[qc], jj);
        if (lane == jj) xr[qc] = xj;
#pragma unroll
        for (int qq = qc; qq < REG_Q; ++qq) {
          if (32 * qq >= len) break;
          const int i = lane + 32 * qq;
          if (i > j && i < len) xr[qq] = fma(-lb[TRI(j, i)], xj, xr[qq]);
        }
      }
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < REG_Q; ++q) {
      const int i = lane + 32 * q;
      if (i < len) x[i] = xr[q];
    }
    __syncwarp();
  }
  // solve U x = b in place (back substitution, column sweep)
  __device__ void trsv_N(const DevModel* M, double* x, int len)
  {
    const double* lb = Lb(M);
    if (len > REG_N) {
      for (int j = len - 1; j >= 0; --j) {
        const double* colj = lb + TRI(0, j);
        double xj = x[j];
        __syncwarp();
        if (xj != 0.0) {
          xj = xj / colj[j];
          for (int i = lane; i < j; i += 32) x[i] -= xj * colj[i];
          if (lane == 0) x[j] = xj;
        }
        __syncwarp();
      }
      return;
    }
    double xr[REG_Q], rd[REG_Q];
#pragma unroll
    for (int q = 0; q < REG_Q; ++q) {
      const int i = lane + 32 * q;
      xr[q] = (i < len) ? x[i] : 0.0;
      rd[q] = 0.0;
      if (32 * q < len) rd[q] = 1.0 / ((i < len) ? lb[TRI(i, i)] : 1.0);
    }
#pragma unroll
    for (int qc = REG_Q - 1; qc >= 0; --qc) {
      if (32 * qc >= len) continue;
      const int jend = min(32, len - 32 * qc);
      for (int jj = jend - 1; jj >= 0; --jj) {
        const int j = 32 * qc + jj;
        const double* colj = lb + TRI(0, j);
        const double xj = __shfl_sync(FULL_MASK, xr[qc] * rd[qc], jj);
        if (lane == jj) xr[qc] = xj;
#pragma unroll
        for (int qq = 0; qq <= qc; ++qq) {
          const int i = lane + 32 * qq;
          if (i < j) xr[qq] = fma(-colj[i], xj, xr[qq]);
        }
      }
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < REG_Q; ++q) {
      const int i = lane + 32 * q;
      if (i < len) x[i] = xr[q];
    }
    __syncwarp();
  }
  // sum of log(L_ii) over lo <= i < hi, one log per lane
  __device__ double sum_log_diag(const DevModel* M, int lo, int hi)
  {
    const double* lb = Lb(M);
    double acc = 0.0;
    for (int i = lo + lane; i < hi; i += 32) acc += flog(lb[TRI(i, i)]);
    return warp_sum_d(acc);
  }
  __device__ double dot(const double* a, const double* b, int len)
  {
    double part = 0.0;
    for (int i = lane; i < len; i += 32) part += a[i] * b[i];
    return warp_sum_d(part);
  }

  /* src/model.hpp:199-237, src/model.hpp:558-576 (Cholesky: LAPACK dpotf2, 'U') */
  __device__ void compute_log_likelihood(DevModel* M)
  {
    int m = M->xcols;
    if (m < 1) {
      if (lane == 0) M->ll = NAN;
      __syncwarp();
      return;
    }
    if (lane == 0) ch->n_lik_full++;
    if (m > SMK) spill(M);
    double* lb = Lb(M);
    double* vb = Vb(M);
    for (int col = 0; col < m; ++col)
      for (int r = lane; r <= col; r += 32) lb[TRI(r, col)] = M->xx[(size_t)col * km + r];
    __syncwarp();
    double log_sum_2 = 0;
    for (int i = lane; i < m; i += 32) {
      lb[TRI(i, i)] += M->inv[i];
      if (i > 0) log_sum_2 += flog(M->inv[i]);
    }
    log_sum_2 = warp_sum_d(log_sum_2);
    __syncwarp();
    double ldq = 0.5 * log_sum_2;
    bool ok = true;
    for (int j = 0; j < m && ok; ++j) {
      double* colj = lb + TRI(0, j);
      double ajj = colj[j] - dot(colj, colj, j);
      if (ajj <= 0.0 || isnan(ajj)) { ok = false; break; }
      ajj = sqrt(ajj);
      __syncwarp();
      if (lane == 0) colj[j] = ajj;
      for (int cc = j + 1 + lane; cc < m; cc += 32) {
        double* colc = lb + TRI(0, cc);
        double t = colc[j];
        for (int q = 0; q < j; ++q) t -= colj[q] * colc[q];
        colc[j] = t / ajj;
      }
      __syncwarp();
    }
    if (lane == 0) {
      M->llen = m;
      M->ldq = ldq;
    }
    __syncwarp();
    if (!ok) {
      if (lane == 0) {
        M->ll = -INFINITY;
        M->syx = INFINITY;
        M->mu_beta_computed = 0;
      }
      __syncwarp();
      return;
    }
    for (int i = lane; i < m; i += 32) vb[i] = M->xy[i];
    __syncwarp();
    trsv_T(M, vb, m);
    double vv = dot(vb, vb, m);
    double ldqx = sum_log_diag(M, 0, m);
    double syx = P.nus2_plus_yy - vv;
    if (lane == 0) {
      M->vlen = m;
      M->syx = syx;
      M->ldqx = ldqx;
      M->ll = ldq - ldqx + P.minus_n_plus_nu_2 * flog(syx);
      M->mu_beta_computed = 0;
    }
    __syncwarp();
  }

  // ------------------------------------------------- genotype products
  // sum_i x_t(g_i) * vec_i for the phenotype (v = 0) or covariate v, in the
  // vector's fixed point, from the per-SNP H and R sums
  __device__ long long geno_dot_fixed(uint32_t snp, int term, int v)
  {
    if (P.gsum) {
      const size_t nv = K.m_e > 1 ? K.m_e : 1;
      const int64_t* g = P.gsum + ((size_t)snp * nv + v) * 2;
      return (long long)coefH(term) * g[0] + (long long)coefR(term) * g[1];
    }
    // the phenotype from the codes (no covariates in this case): 16
    // individuals per 32-bit word, the phenotype is zero outside the sample
    if (helpers) {
      if (lane == 0) {
        s.job_kind = HJ_XY;
        s.job_snp = snp;
        s.job_term = term;
      }
      __syncwarp();
      bar_sync_all();
      const long long a = warp_sum_ll(geno_dot_part(K, P, snp, term, threadIdx.x, BMG_MOVE_THREADS));
      if (lane == 0) s.job_part[0] = a;
      bar_sync_all();
      long long t = 0;
      for (int w = 0; w < BMG_MOVE_THREADS / 32; ++w) t += s.job_part[w];
      __syncwarp();
      return t;
    }
    return warp_sum_ll(geno_dot_part(K, P, snp, term, lane, 32));
  }
  // exact sum_i x_t(g_a,i) x_u(g_b,i) from the 2-bit codes
  __device__ long long geno_cross(uint32_t a, int t, uint32_t b, int u)
  {
    if (a == b) return term_cross_same(P.cnt, a, t, u);
    const uint64_t* ra = (const uint64_t*)(K.geno + (size_t)a * K.gs);
    const uint64_t* rb = (const uint64_t*)(K.geno + (size_t)b * K.gs);
    unsigned nw64 = K.gs / 8;
    long long hh = 0, hr = 0, rh = 0, rr = 0;
    const uint64_t m5 = 0x5555555555555555ull;
    for (unsigned w = lane; w < nw64; w += 32) {
      uint64_t x = ra[w], y = rb[w];
      const uint64_t mk = P.mask2 ? P.mask2[w] : m5;
      uint64_t xh = (x >> 1) & mk, xl = x & m5, yh = (y >> 1) & mk, yl = y & m5;
      uint64_t Hx = xh & ~xl, Rx = xh & xl, Hy = yh & ~yl, Ry = yh & yl;
      hh += __popcll(Hx & Hy);
      hr += __popcll(Hx & Ry);
      rh += __popcll(Rx & Hy);
      rr += __popcll(Rx & Ry);
    }
    long long v = (long long)coefH(t) * coefH(u) * hh + (long long)coefH(t) * coefR(u) * hr +
                  (long long)coefR(t) * coefH(u) * rh + (long long)coefR(t) * coefR(u) * rr;
    return warp_sum_ll(v);
  }
  // X' column entry between model column r and a new genotype column (snp, term)
  __device__ double cross_col(const DevModel* M, int r, uint32_t snp, int term)
  {
    if (r < (int)K.m_e) {
      if (r == 0) return (double)term_sum(P.cnt, snp, term);
      long long acc = geno_dot_fixed(snp, term, r);
      return (double)acc * ldexp(1.0, -K.se[r]);
    }
    return (double)geno_cross(M->xc_snp[r], M->xc_type[r], snp, term);
  }
  // The same for the genotype columns r0 <= r < r1: on all eight warps while
  // they help warp 0 (a move), else on warp 0 alone
  __device__ void cross_cols(const DevModel* M, int r0, int r1, uint32_t snp, int term, double* out)
  {
    if (r1 <= r0) return;
    if (helpers) {
      if (lane == 0) {
        s.job_kind = HJ_CROSS;
        s.job_M = M;
        s.job_r0 = r0;
        s.job_r1 = r1;
        s.job_snp = snp;
        s.job_term = term;
        s.job_out = out;
      }
      __syncwarp();
      bar_sync_all();
      cross_cols_part(K, P, M, r0, r1, snp, term, out, 0, BMG_MOVE_THREADS / 32);
      bar_sync_all();
      return;
    }
    cross_cols_part(K, P, M, r0, r1, snp, term, out, 0, 1);
  }
  // end of the helpers' service (warp 0, after a move)
  __device__ void help_exit()
  {
    if (!helpers) return;
    if (lane == 0) s.job_kind = HJ_EXIT;
    __syncwarp();
    bar_sync_all();
    helpers = false;
  }

  // ------------------------------------------------------ missing calls
  // The codes hold a missing call as 01, which every product above reads as
  // 0; the chain's imputed values (K.miss_val, the reference's DataModel
  // overlay, src/data_model.cpp:30-72) enter through the corrections below.
  __device__ bool has_miss(uint32_t snp) const { return K.miss_total && K.miss_off[snp + 1] > K.miss_off[snp]; }
  __device__ int code_g(uint32_t snp, uint32_t i) const
  {
    const int code = (K.geno[(size_t)snp * K.gs + (i >> 2)] >> (2 * (i & 3))) & 3;
    return code == 2 ? 1 : (code == 3 ? 2 : 0);
  }
  // position of individual i among the SNP's missing calls, or -1
  __device__ long long miss_pos(uint32_t snp, uint32_t i) const
  {
    long long lo = K.miss_off[snp], hi = K.miss_off[snp + 1];
    while (lo < hi) {
      const long long mid = (lo + hi) >> 1;
      if (K.miss_ind[mid] < i) lo = mid + 1;
      else hi = mid;
    }
    return (lo < K.miss_off[snp + 1] && K.miss_ind[lo] == i) ? lo : -1;
  }
  __device__ int mval(long long pos) const { return K.miss_val[(size_t)c * K.miss_total + pos]; }
  // genotype of SNP snp at individual i with the chain's imputed values
  __device__ int geno_imp(uint32_t snp, uint32_t i) const
  {
    const long long q = has_miss(snp) ? miss_pos(snp, i) : -1;
    return q >= 0 ? mval(q) : code_g(snp, i);
  }
  /* DataModel::sample_missing_single (src/data_model.cpp:92-103): fresh
     imputed values for a SNP's missing calls, one uniform each in call order */
  __device__ void draw_missing(uint32_t snp)
  {
    const long long o0 = K.miss_off[snp], nm = K.miss_off[snp + 1] - o0;
    const double* mp = K.miss_prior + 3 * (size_t)snp;
    for (long long q = lane; q < nm; q += 32)
      K.miss_val[(size_t)c * K.miss_total + o0 + q] =
          (uint8_t)miss_draw(mp, bmg_uniform01_at(rng.key0, rng.key1, rng.slot + (uint64_t)q));
    rng.slot += (uint64_t)nm;
    __syncwarp();
  }
  // what the missing calls of SNPs a (term t) and b (term u) add to x_t(a)'
  // x_u(b) over the product with the missing calls read as 0
  __device__ long long cross_corr(uint32_t a, int t, uint32_t b, int u) const
  {
    long long acc = 0;
    if (has_miss(a)) {
      for (long long q = K.miss_off[a] + lane; q < K.miss_off[a + 1]; q += 32) {
        const uint32_t i = K.miss_ind[q];
        acc += gval_term(mval(q), t) * gval_term(a == b ? mval(q) : geno_imp(b, i), u);
      }
    }
    if (has_miss(b) && a != b) {
      for (long long q = K.miss_off[b] + lane; q < K.miss_off[b + 1]; q += 32) {
        const uint32_t i = K.miss_ind[q];
        if (has_miss(a) && miss_pos(a, i) >= 0) continue;  // counted above
        acc += gval_term(code_g(a, i), t) * gval_term(mval(q), u);
      }
    }
    return warp_sum_ll(acc);
  }
  // ... and to x_t(snp)' v for the fixed-point vector v (y: yint; covariate r: eint)
  __device__ long long vec_corr(uint32_t snp, int t, const int64_t* v) const
  {
    long long acc = 0;
    for (long long q = K.miss_off[snp] + lane; q < K.miss_off[snp + 1]; q += 32)
      acc += (long long)gval_term(mval(q), t) * v[K.miss_ind[q]];
    return warp_sum_ll(acc);
  }
  __device__ long long sum_corr(uint32_t snp, int t) const
  {
    long long acc = 0;
    for (long long q = K.miss_off[snp] + lane; q < K.miss_off[snp + 1]; q += 32) acc += gval_term(mval(q), t);
    return warp_sum_ll(acc);
  }

  // --------------------------------------------------------- model updates
  /* src/model.hpp:432-506 with src/symmmatrix.cpp:144-164 */
  __device__ void upd_add(DevModel* M, uint32_t snp, int mi, int term, bool is2, double invv, bool update)
  {
    int col = M->xcols;
    if (col + 1 > SMK) spill(M);
    if (lane == 0) {
      if (is2) M->x_ind2[mi] = col;
      else { M->x_ind1[mi] = col; M->x_ind2[mi] = 0; }
      M->xc_snp[col] = snp;
      M->xc_type[col] = term;
      M->xcols = col + 1;
      M->inv[col] = invv;
    }
    long long xyi = geno_dot_fixed(snp, term, 0);
    const bool miss = has_miss(snp);
    if (miss) xyi += vec_corr(snp, term, P.yint);
    double xyc = (double)xyi * ldexp(1.0, -P.sy);
    __syncwarp();
    if (lane == 0) M->xy[col] = xyc;
    double* xxcol = &M->xx[(size_t)col * km];
    const int me = min((int)K.m_e, col);
    for (int r = 0; r < me; ++r) {
      double v = cross_col(M, r, snp, term);
      if (miss) {
        if (r == 0) v += (double)sum_corr(snp, term);
        else v = (double)(geno_dot_fixed(snp, term, r) + vec_corr(snp, term, K.eint + (size_t)r * K.n)) *
                 ldexp(1.0, -K.se[r]);
      }
      if (lane == 0) xxcol[r] = v;
    }
    cross_cols(M, me, col, snp, term, xxcol);
    long long self = term_cross_same(P.cnt, snp, term, term);
    if (K.miss_total) {
      // the missing calls of the new SNP and of the model's SNPs
      for (int r = me; r < col; ++r) {
        const uint32_t sr = M->xc_snp[r];
        if (!miss && !has_miss(sr)) continue;
        const long long d = cross_corr(sr, M->xc_type[r], snp, term);
        __syncwarp();
        if (lane == 0) xxcol[r] += (double)d;
        __syncwarp();
      }
      if (miss) self += cross_corr(snp, term, snp, term);
    }
    if (lane == 0) xxcol[col] = (double)self;
    __syncwarp();
    if (!update) {
      if (lane == 0) { M->llen = col + 1; M->vlen = col + 1; }
      __syncwarp();
      return;
    }
    if (lane == 0) ch->n_lik_add++;
    double* lcol = Lb(M) + TRI(0, col);
    for (int r = lane; r <= col; r += 32) lcol[r] = xxcol[r];
    __syncwarp();
    trsv_T(M, lcol, col);
    double lmm2 = xxcol[col] + invv - dot(lcol, lcol, col);
    if (lane == 0) M->llen = col + 1;
    __syncwarp();
    if (lmm2 <= 0) {
      if (lane == 0) {
        M->ll = -INFINITY;
        M->syx = INFINITY;
        M->mu_beta_computed = 0;
        M->vlen = col + 1;
      }
      __syncwarp();
      return;
    }
    double lcc = sqrt(lmm2);
    double* vb = Vb(M);
    double vm2 = M->xy[col] - dot(lcol, vb, col);
    double vc = vm2 / lcc;
    double syx = M->syx - vc * vc;
    double ldq = M->ldq + 0.5 * flog(invv);
    double ldqx = M->ldqx + flog(lcc);
    __syncwarp();
    if (lane == 0) {
      lcol[col] = lcc;
      M->vlen = col + 1;
      vb[col] = vc;
      M->syx = syx;
      M->ldq = ldq;
      M->ldqx = ldqx;
      M->ll = ldq - ldqx + P.minus_n_plus_nu_2 * flog(syx);
    }
    __syncwarp();
  }

  /* src/model.hpp:239-268 */
  __device__ void add_term(DevModel* M, uint32_t snp, int t_ind, const double* itv)
  {
    int type = K.types[t_ind];
    bool ah = (type == 4);
    int mi = M->k;
    if (M->xcols + 1 + (ah ? 1 : 0) > (int)km) { fail(BMG_DERR_CAPACITY); return; }
    if (lane == 0) {
      M->loci[mi] = snp;
      M->Ns[type]++;
      M->type_inds[mi] = (uint8_t)t_ind;
      M->k = mi + 1;
      M->mu_beta_computed = 0;
    }
    __syncwarp();
    if (ah) {
      upd_add(M, snp, mi, 0, false, itv[0], true);
      if (isfinite(M->syx)) upd_add(M, snp, mi, 1, true, itv[1], true);
    } else {
      upd_add(M, snp, mi, type, false, itv[0], true);
    }
  }

  // remove element `at` of an array of length len (warp)
  template <class T>
  __device__ void erase(T* a, int len, int at)
  {
    for (int base = at; base < len - 1; base += 32) {
      int i = base + lane;
      T v = (i < len - 1) ? a[i + 1] : T();
      __syncwarp();
      if (i < len - 1) a[i] = v;
      __syncwarp();
    }
  }

  /* src/dchex.f:130-220 (job 2) on L with k = x_ind + 1, l = p = order:
     column k moves to the end and the left shift's subdiagonal is removed by
     Givens rotations.  Rotation ii acts on rows k + ii - 1 and k + ii of
     every later column and is made from column k + ii - 1 once that column
     has taken rotations 1 .. ii - 1.  Here lane t holds column k + t and the
     rotations run as a wavefront (lane t applies rotation q of its group at
     step t + q and makes its own at step 2t + 1), 32 columns at a time, so
     the chain of FP64 instructions grows with the order instead of its
     square.  Each element takes the reference's rotations in the reference's
     order; the rotations come from the same inputs, formed with one
     reciprocal square root instead of dchex's scaled divisions. */
  __device__ void dchex_left(DevModel* M, int x_ind, int order, double* cs, double* sn)
  {
    if (order <= SMK) { cs = s.cs; sn = s.sn; }
    const int k = x_ind + 1, l = order;
    const int km1 = k - 1, lmk = l - k;
    double* r = Lb(M);
#define R_(i, j) r[TRI((i) - 1, (j) - 1)]
    // column k is kept aside at sn[lmk ..], the columns after it move left
    // and their diagonals, now below the diagonal, wait in sn[0 .. lmk - 1]
    for (int i = 1 + lane; i <= k; i += 32) sn[lmk + i - 1] = R_(i, k);
    __syncwarp();
    for (int j = k; j <= l - 1; ++j) {
      // column j's slots end where column j + 1's begin: the copy never
      // overwrites a source element
      for (int i = 1 + lane; i <= j; i += 32) R_(i, j) = R_(i, j + 1);
      if (lane == 0) sn[j - km1 - 1] = R_(j + 1, j + 1);
      __syncwarp();
    }
    for (int i = 1 + lane; i <= k; i += 32) R_(i, l) = sn[lmk + i - 1];
    for (int i = k + 1 + lane; i <= l; i += 32) R_(i, l) = 0.0;
    __syncwarp();
    const int ncols = l - k + 1;  // columns k .. l
    for (int g0 = 0; g0 < ncols; g0 += 32) {
      const int t = g0 + lane;
      const bool mine = t < ncols;
      const int j = k + t;
      // rotations of earlier groups, in order
      for (int rr = 1; rr <= g0; ++rr) {
        if (mine) {
          const double c = cs[rr - 1], sg = sn[rr - 1];
          const int i = k + rr - 1;
          const double a = R_(i, j), bb = R_(i + 1, j);
          R_(i + 1, j) = c * bb - sg * a;
          R_(i, j) = c * a + sg * bb;
        }
      }
      __syncwarp();
      for (int step = 1; step < 64; ++step) {
        const int q = step - lane;
        const int rr = g0 + q;
        if (mine && q >= 1) {
          if (rr <= t && rr <= lmk) {
            const double c = cs[rr - 1], sg = sn[rr - 1];
            const int i = k + rr - 1;
            const double a = R_(i, j), bb = R_(i + 1, j);
            R_(i + 1, j) = c * bb - sg * a;
            R_(i, j) = c * a + sg * bb;
          } else if (rr == t + 1 && j < l) {
            // drotg(r(j,j), s(jj)): r takes the sign of the larger input
            const double sa = R_(j, j), sb = sn[rr - 1];
            const double h2 = sa * sa + sb * sb;
            double rv = 0.0, c = 1.0, sg = 0.0;
            if (h2 > 0.0) {
              const double sgn = (fabs(sa) > fabs(sb) ? sa : sb) < 0.0 ? -1.0 : 1.0;
              const double ri = rsqrt(h2) * sgn;
              rv = h2 * ri;
              c = sa * ri;
              sg = sb * ri;
            }
            R_(j, j) = rv;
            cs[rr - 1] = c;
            sn[rr - 1] = sg;
          }
        }
        __syncwarp();
      }
    }
#undef R_
    __syncwarp();
  }

  /* src/model.hpp:508-556 with src/symmmatrix.cpp:126-195 */
  __device__ void upd_rem(DevModel* M, int x_ind, double* cs, double* sn)
  {
    int len = M->xcols;
    double invv = M->inv[x_ind];
    __syncwarp();
    erase(M->xc_snp, len, x_ind);
    erase(M->xc_type, len, x_ind);
    erase(M->xy, len, x_ind);
    erase(M->inv, len, x_ind);
    // xx.remove_colrow
    for (int i = x_ind; i < len - 1; ++i) {
      for (int j = lane; j <= i; j += 32) {
        double v = (j < x_ind) ? M->xx[(size_t)(i + 1) * km + j] : M->xx[(size_t)(i + 1) * km + j + 1];
        M->xx[(size_t)i * km + j] = v;
      }
      __syncwarp();
    }
    int xc = len - 1;
    if (lane == 0) { M->xcols = xc; ch->n_lik_rem++; }
    __syncwarp();
    if (x_ind == xc) {
      double lxx = L(M, x_ind, x_ind);
      double vx = Vb(M)[x_ind];
      double ldqx = M->ldqx - flog(lxx);
      double syx = M->syx + vx * vx;
      __syncwarp();
      if (lane == 0) {
        M->ldqx = ldqx;
        M->syx = syx;
        M->llen = xc;
        M->vlen = xc;
      }
      __syncwarp();
    } else {
      int order = M->llen;
      dchex_left(M, x_ind, order, cs, sn);
      int nl = order - 1;
      // rows whose diagonal came out negative change sign (a sign flip, the
      // reference's multiplication by -1); the diagonal tests are lane-parallel
      for (int base = x_ind; base < nl; base += 32) {
        const int i0 = base + lane;
        unsigned neg = __ballot_sync(FULL_MASK, i0 < nl && L(M, i0, i0) < 0);
        while (neg) {
          const int i = base + __ffs(neg) - 1;
          neg &= neg - 1;
          for (int j = i + lane; j < nl; j += 32) {
            double& e = L(M, i, j);
            e = __longlong_as_double(__double_as_longlong(e) ^ (long long)0x8000000000000000ull);
          }
          __syncwarp();
        }
      }
      double* vb = Vb(M);
      for (int i = lane; i < xc; i += 32) vb[i] = M->xy[i];
      __syncwarp();
      trsv_T(M, vb, nl);
      double ldqx = sum_log_diag(M, 0, nl);
      double syx = P.nus2_plus_yy - dot(vb, vb, xc);
      if (lane == 0) {
        M->llen = nl;
        M->vlen = xc;
        M->ldqx = ldqx;
        M->syx = syx;
      }
      __syncwarp();
    }
    double ldq = M->ldq - 0.5 * flog(invv);
    double ll = ldq - M->ldqx + P.minus_n_plus_nu_2 * flog(M->syx);
    __syncwarp();
    if (lane == 0) {
      M->ldq = ldq;
      M->ll = ll;
    }
    __syncwarp();
  }

  /* src/model.hpp:270-312 */
  __device__ void remove_term(DevModel* M, int mi, double* cs, double* sn)
  {
    int type = K.types[M->type_inds[mi]];
    int xi1 = M->x_ind1[mi], xi2 = M->x_ind2[mi];
    int k = M->k;
    __syncwarp();
    if (lane == 0) M->Ns[type]--;
    erase(M->loci, k, mi);
    erase(M->type_inds, k, mi);
    erase(M->x_ind1, k, mi);
    erase(M->x_ind2, k, mi);
    int xmove = (type == 4) ? 2 : 1;
    for (int i = mi + lane; i < k - 1; i += 32) {
      M->x_ind1[i] -= xmove;
      M->x_ind2[i] -= xmove;
    }
    if (lane == 0) M->k = k - 1;
    __syncwarp();
    if (type == 4) {
      if (xi1 > xi2) { upd_rem(M, xi1, cs, sn); upd_rem(M, xi2, cs, sn); }
      else { upd_rem(M, xi2, cs, sn); upd_rem(M, xi1, cs, sn); }
    } else {
      upd_rem(M, xi1, cs, sn);
    }
    if (lane == 0) M->mu_beta_computed = 0;
    __syncwarp();
  }

  // model index of a SNP in a model (linear search; -1 if absent)
  __device__ int find_locus(const DevModel* M, uint32_t snp)
  {
    int found = -1;
    for (int base = 0; base < M->k; base += 32) {
      int i = base + lane;
      bool hit = (i < M->k) && (M->loci[i] == snp);
      unsigned b = __ballot_sync(FULL_MASK, hit);
      if (b) { found = base + __ffs(b) - 1; break; }
    }
    return found;
  }

  /* Sampler::sample_missing (src/sampler.cpp:264-453): the missing calls of
     the model's SNPs are drawn from their conditional given the residuals, SNP
     by SNP in model order (one uniform per call, in call order; the calls of
     one SNP are distinct individuals, so they are drawn lane-parallel), then
     X'y and X'X of the changed columns are formed again from the codes and
     the new values.  The reference's r^2 term cancels from the normalised
     weights and is left out. */
  __device__ void sample_missing_gibbs()
  {
    DevModel* M = cur;
    if (!K.miss_total) return;
    const double s2x2 = M->sigma2 * 2;
    const int ncols = min(M->blen, M->xcols);
    bool any = false;
    for (int li = 0; li < M->k; ++li) {
      const uint32_t ind = M->loci[li];
      if (!has_miss(ind)) continue;
      any = true;
      const int type = K.types[M->type_inds[li]];
      const int ct = (type == 4) ? 0 : type;  // the coding of the first column
      const int x1 = M->x_ind1[li], x2 = (type == 4) ? (int)M->x_ind2[li] : 0;
      const double b1 = M->beta[x1], b2 = (type == 4) ? M->beta[x2] : 0.0;
      const double* mp = K.miss_prior + 3 * (size_t)ind;
      const double lp1 = flog(mp[1] - mp[0]) - flog(mp[0]), lp2 = flog(mp[2] - mp[1]) - flog(mp[0]);
      const long long o0 = K.miss_off[ind], nmc = K.miss_off[ind + 1] - o0;
      for (long long q = lane; q < nmc; q += 32) {
        const uint32_t im = K.miss_ind[o0 + q];
        double yh = 0.0;
        for (int col = 0; col < ncols; ++col) {
          double xv;
          if (col < (int)K.m_e) xv = (col == 0) ? 1.0 : K.e[(size_t)col * K.n + im];
          else xv = (double)gval_term(geno_imp(M->xc_snp[col], im), M->xc_type[col]);
          yh = fma(M->beta[col], xv, yh);
        }
        const double res = P.y[im] - yh;
        const int cv = mval(o0 + q);
        const double t1 = gval_term(cv, ct), t2 = (cv == 1);
        double nt[3];
        for (int k = 0; k < 3; ++k) {
          nt[k] = res - b1 * (gval_term(k, ct) - t1);
          if (type == 4) nt[k] -= b2 * ((k == 1) - t2);
        }
        const double l1 = lp1 - (nt[1] * nt[1] - nt[0] * nt[0]) / s2x2;
        const double l2 = lp2 - (nt[2] * nt[2] - nt[0] * nt[0]) / s2x2;
        const double c1 = exp(l1) + 1.0;
        const double c2 = exp(l2) + c1;
        const double r = bmg_uniform01_at(rng.key0, rng.key1, rng.slot + (uint64_t)q) * c2;
        K.miss_val[(size_t)c * K.miss_total + o0 + q] = (uint8_t)(r < 1.0 ? 0 : (r < c1 ? 1 : 2));
      }
      rng.slot += (uint64_t)nmc;
      __syncwarp();
    }
    if (!any) return;
    // X'y and X'X of the columns of SNPs with missing calls, exact
    const int xc = M->xcols, me = K.m_e;
    for (int xi = me; xi < xc; ++xi) {
      const uint32_t snp = M->xc_snp[xi];
      if (!has_miss(snp)) continue;
      const int t = M->xc_type[xi];
      const long long xyi = geno_dot_fixed(snp, t, 0) + vec_corr(snp, t, P.yint);
      __syncwarp();
      if (lane == 0) M->xy[xi] = (double)xyi * ldexp(1.0, -P.sy);
      for (int r = 0; r < xc; ++r) {
        double v;
        if (r < me) {
          if (r == 0) v = (double)(term_sum(P.cnt, snp, t) + sum_corr(snp, t));
          else v = (double)(geno_dot_fixed(snp, t, r) + vec_corr(snp, t, K.eint + (size_t)r * K.n)) *
                   ldexp(1.0, -K.se[r]);
        } else {
          const uint32_t sr = M->xc_snp[r];
          const int tr = M->xc_type[r];
          v = (double)(geno_cross(sr, tr, snp, t) + cross_corr(sr, tr, snp, t));
        }
        __syncwarp();
        if (lane == 0) M->xx[(size_t)max(r, xi) * km + min(r, xi)] = v;
        __syncwarp();
      }
    }
    if (lane == 0) M->mu_beta_computed = 0;
    __syncwarp();
  }

  /* src/model.hpp:314-342, src/rand.hpp:144-168 */
  __device__ void sample_beta_sigma2(DevModel* M)
  {
    double s2 = sinvchi2(M->syx / P.n_plus_nu);
    int len = M->vlen;
    // the triangular solves run on shared copies when the model fits
    const bool on_chip = len <= SMK && M->llen <= SMK;
    double* mu = on_chip ? s.tv[0] : M->mu_beta;
    double* bt = on_chip ? s.tv[1] : M->beta;
    if (!M->mu_beta_computed) {
      const double* vb = Vb(M);
      for (int i = lane; i < len; i += 32) mu[i] = vb[i];
      __syncwarp();
      trsv_N(M, mu, M->llen);
      if (lane == 0) M->mu_beta_computed = 1;
    } else if (on_chip) {
      for (int i = lane; i < len; i += 32) mu[i] = M->mu_beta[i];
    }
    // normal i of the vector is the chain's draw at slot + i
    for (int i = lane; i < len; i += 32) bt[i] = bmg_normal_at(rng.key0, rng.key1, rng.slot + i);
    rng.slot += len;
    __syncwarp();
    trsv_N(M, bt, M->llen);
    double sc = sqrt(s2);
    for (int i = lane; i < len; i += 32) {
      M->beta[i] = sc * bt[i] + mu[i];
      if (on_chip) M->mu_beta[i] = mu[i];
    }
    if (lane == 0) {
      M->sigma2 = s2;
      M->blen = len;
    }
    __syncwarp();
  }

  /* src/prior.cpp:71-114 */
  __device__ void sample_tau2(DevModel* M)
  {
    double a2s2 = ch->alpha2 * M->sigma2;
    int me = K.m_e, bl = M->blen;
    if (K.use_individual_tau2) {
      for (int i = me; i < bl; ++i) {
        int t = M->xc_type[i];
        double nu = K.nu_tau2[t] + 1.0;
        double b = M->beta[i];
        double s2 = (P.nus2_tau2[t] + b * b / a2s2) / nu;
        double v = 1.0 / (ch->alpha2 * sinvchi2(nu, s2));
        __syncwarp();
        if (lane == 0) M->inv[i] = v;
      }
    } else {
      double b2s[4] = {0, 0, 0, 0};
      int mt[4] = {0, 0, 0, 0};
      for (int i = me; i < bl; ++i) {
        int t = M->xc_type[i];
        b2s[t] += M->beta[i] * M->beta[i];
        ++mt[t];
      }
      double it[4];
      for (int t = 0; t < 4; ++t) {
        it[t] = ch->inv_t2a2[t];
        if (!K.allow_terms[t]) continue;
        double nu = K.nu_tau2[t] + mt[t];
        double s2 = (P.nus2_tau2[t] + b2s[t] / a2s2) / nu;
        it[t] = 1.0 / (ch->alpha2 * sinvchi2(nu, s2));
      }
      __syncwarp();
      if (lane == 0)
        for (int t = 0; t < 4; ++t) ch->inv_t2a2[t] = it[t];
      for (int i = me + lane; i < bl; i += 32) M->inv[i] = it[M->xc_type[i]];
    }
    if (lane == 0) M->mu_beta_computed = 0;
    __syncwarp();
  }

  /* src/prior.cpp:116-141 */
  __device__ void set_alpha(double val, DevModel* M)
  {
    double old2 = ch->alpha2;
    double a2 = val * val;
    int me = K.m_e, bl = M->blen;
    __syncwarp();
    if (K.use_individual_tau2) {
      for (int i = me + lane; i < bl; i += 32) M->inv[i] = M->inv[i] * old2 / a2;
    } else {
      double it[4];
      for (int t = 0; t < 4; ++t) it[t] = K.allow_terms[t] ? ch->inv_t2a2[t] * old2 / a2 : ch->inv_t2a2[t];
      __syncwarp();
      if (lane == 0)
        for (int t = 0; t < 4; ++t) ch->inv_t2a2[t] = it[t];
      for (int i = me + lane; i < bl; i += 32) M->inv[i] = it[M->xc_type[i]];
    }
    if (lane == 0) { ch->alpha = val; ch->alpha2 = a2; }
    __syncwarp();
  }

  /* src/prior.cpp:30-69; xbxb and ebxb come from the bulk phase */
  __device__ double sample_alpha(DevModel* M, double xbxb, double ebxb)
  {
    int nterms = M->blen - (int)K.m_e;
    double a = ch->alpha;
    for (int t = 0; t < 64; ++t) {
      if (nterms > 0) {
        if ((a <= 0.0) || flog(u01()) <= -2.0 * K.mu_alpha * a) a = -a;
        double as2 = a * M->sigma2;
        double var = 1.0 / (1.0 + xbxb / (a * as2));
        double mu = var * (K.mu_alpha - ebxb / as2);
        a = sqrt(var) * nrm() + mu;
      } else {
        a = nrm() + K.mu_alpha;
      }
      if (!(a == 0 || a * a == 0)) break;
    }
    if (lane == 0) M->mu_beta_computed = 0;
    __syncwarp();
    return a;
  }

  // --------------------------------------------------------- proposals
  __device__ bool pend_find(uint32_t snp, int* at) const
  {
    int found = -1;
    for (int base = 0; base < s.n_pend; base += 32) {
      int i = base + lane;
      bool hit = (i < s.n_pend) && (s.pend_snp[i] == (int)snp);
      unsigned b = __ballot_sync(FULL_MASK, hit);
      if (b) { found = base + __ffs(b) - 1; break; }
    }
    *at = found;
    return found >= 0;
  }
  __device__ bool base_zero(uint32_t snp) const
  {
    return (K.basebits[(size_t)c * ((K.p + 31) / 32) + (snp >> 5)] >> (snp & 31)) & 1u;
  }
  // dd_add zero state toggles (src/discrete_distribution.hpp:156-199)
  __device__ void add_set_zero(uint32_t snp, bool zero)
  {
    int at;
    bool in_list = pend_find(snp, &at);
    bool zeroed = base_zero(snp) != in_list;
    if (zeroed == zero) return;
    if (K.lrn.on) {
      const long long wm = mlp_wint(snp);
      __syncwarp();
      if (lane == 0) s.w_m += zero ? -wm : wm;
    }
    if (in_list) {
      int last = s.n_pend - 1;
      __syncwarp();
      if (lane == 0) {
        s.pend_snp[at] = s.pend_snp[last];
        s.pend_pos[at] = s.pend_pos[last];
        s.pend_d[at] = s.pend_d[last];
        s.n_pend = last;
      }
    } else {
      if (s.n_pend >= BMG_PEND_MAX) { fail(BMG_DERR_PEND); return; }
      long long w = qadd_int(snp);
      __syncwarp();
      if (lane == 0) {
        int i = s.n_pend;
        s.pend_snp[i] = (int)snp;
        s.pend_pos[i] = K.pos[snp];
        s.pend_d[i] = base_zero(snp) ? w : -w;
        s.n_pend = i + 1;
      }
    }
    __syncwarp();
  }
  __device__ long long add_total_int()
  {
    long long t = 0;
    for (int i = lane; i < s.n_pend; i += 32) t += s.pend_d[i];
    return ch->cadd_total + warp_sum_ll(t);
  }
  __device__ double add_total() { return (double)add_total_int() * ldexp(1.0, -K.qs); }

  // ---- learned part of the add proposal: candidate weights in fixed point
  // (x 2^40, exact sums), zero for SNPs outside the chain's candidate table
  __device__ long long mlp_wint(uint32_t snp) const
  {
    const uint32_t T = K.lrn.topk, n = K.lrn.t_n[c];
    const uint32_t* ts = K.lrn.t_snp + (size_t)c * T;
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (ts[mid] < snp) lo = mid + 1;
      else hi = mid;
    }
    return (lo < n && ts[lo] == snp) ? __double2ll_rn(K.lrn.t_s[(size_t)c * T + lo] * 0x1p40) : 0ll;
  }
  // at a launch's start the zero set is the current model
  __device__ void mlp_init_total()
  {
    const uint32_t T = K.lrn.topk, n = K.lrn.t_n[c];
    long long w = 0;
    for (uint32_t i = lane; i < n; i += 32) w += __double2ll_rn(K.lrn.t_s[(size_t)c * T + i] * 0x1p40);
    w = warp_sum_ll(w);
    for (int i = 0; i < cur->k; ++i) w -= mlp_wint(cur->loci[i]);
    __syncwarp();
    if (lane == 0) s.w_m = w;
    __syncwarp();
  }
  __device__ bool pend_has(uint32_t snp) const
  {
    for (int i = 0; i < s.n_pend; ++i)
      if (s.pend_snp[i] == (int)snp) return true;
    return false;
  }
  // a candidate outside the zero set, with probability proportional to its weight
  __device__ uint32_t mlp_sample(long long wm)
  {
    long long target = (long long)floor(u01() * (double)wm);
    if (target >= wm) target = wm - 1;
    const uint32_t T = K.lrn.topk, n = K.lrn.t_n[c];
    const uint32_t* ts = K.lrn.t_snp + (size_t)c * T;
    const uint32_t per = (n + 31) / 32, i0 = min(n, lane * per), i1 = min(n, i0 + per);
    long long mine = 0;
    for (uint32_t i = i0; i < i1; ++i)
      if (base_zero(ts[i]) == pend_has(ts[i])) mine += __double2ll_rn(K.lrn.t_s[(size_t)c * T + i] * 0x1p40);
    long long incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
      const long long v = __shfl_up_sync(FULL_MASK, incl, o);
      if (lane >= o) incl += v;
    }
    const unsigned hit = __ballot_sync(FULL_MASK, incl > target);
    const int src = hit ? __ffs(hit) - 1 : 31;
    uint32_t pick = 0xFFFFFFFFu, last = 0xFFFFFFFFu;
    if (lane == src) {
      long long run = incl - mine;
      for (uint32_t i = i0; i < i1; ++i) {
        if (base_zero(ts[i]) != pend_has(ts[i])) continue;
        last = ts[i];
        run += __double2ll_rn(K.lrn.t_s[(size_t)c * T + i] * 0x1p40);
        if (run > target) { pick = ts[i]; break; }
      }
      if (pick == 0xFFFFFFFFu) pick = last;
    }
    return __shfl_sync(FULL_MASK, pick, src);
  }

  // C'(q): weight of in-order positions < q after the pending flips
  __device__ long long cum_at(long long q) const
  {
    long long v = K.cadd[(size_t)c * (K.p + 1) + q];
    for (int i = 0; i < s.n_pend; ++i)
      if (s.pend_pos[i] < q) v += s.pend_d[i];
    return v;
  }
  /* src/discrete_distribution.hpp:125-153 on the in-order prefix */
  __device__ uint32_t add_sample()
  {
    long long totali = add_total_int();
    double total = (double)totali * ldexp(1.0, -K.qs);
    double r = u01() * total;
    double scale = ldexp(1.0, -K.qs);
    long long lo = 0, hi = (long long)K.p;
    for (int it = 0; it < 16 && hi - lo > 1; ++it) {
      long long span = hi - lo;
      long long step = (span + 31) / 32;
      long long q = lo + (long long)lane * step;
      bool ok = false;
      if (q < hi) ok = ((double)cum_at(q) * scale) <= r;
      unsigned b = __ballot_sync(FULL_MASK, ok);
      int last = 31 - __clz(b);  // lane 0 always satisfies (C'(lo) <= r)
      lo = lo + (long long)last * step;
      hi = min(hi, lo + step);
    }
    // guard against rounding at the top: step back to a position with weight
    long long q = lo;
    for (int t = 0; t < 64 && q > 0; ++t) {
      long long w = cum_at(q + 1) - cum_at(q);
      if (w > 0) break;
      --q;
    }
    return (uint32_t)K.inv[q];
  }

  // dd_rem set (src/discrete_distribution.hpp semantics on the few non-zero SNPs)
  __device__ void rs_build_from(const DevModel* M)
  {
    int k = M->k;
    if (k > BMG_REMSET_MAX - 2 * BMG_MAX_MS) { fail(BMG_DERR_REMSET); return; }
    // rank by in-order position (positions are distinct)
    for (int i = lane; i < k; i += 32) {
      uint32_t si = M->loci[i];
      int pi = K.pos[si];
      int rank = 0;
      for (int j = 0; j < k; ++j) rank += (K.pos[M->loci[j]] < pi);
      s.rs_snp[rank] = si;
      s.rs_pos[rank] = pi;
      s.rs_w[rank] = qrem(si);
      s.rs_on[rank] = 1;
    }
    if (lane == 0) s.n_rs = k;
    __syncwarp();
  }
  __device__ void rs_set(uint32_t snp, bool on)
  {
    int n = s.n_rs;
    int found = -1;
    for (int base = 0; base < n; base += 32) {
      int i = base + lane;
      bool hit = (i < n) && (s.rs_snp[i] == snp);
      unsigned b = __ballot_sync(FULL_MASK, hit);
      if (b) { found = base + __ffs(b) - 1; break; }
    }
    if (found >= 0) {
      __syncwarp();
      if (lane == 0) s.rs_on[found] = on ? 1 : 0;
      __syncwarp();
      return;
    }
    if (!on) return;
    if (n >= BMG_REMSET_MAX) { fail(BMG_DERR_REMSET); return; }
    int p = K.pos[snp];
    double w = qrem(snp);
    __syncwarp();
    if (lane == 0) {
      int i = n;
      while (i > 0 && s.rs_pos[i - 1] > p) {
        s.rs_snp[i] = s.rs_snp[i - 1];
        s.rs_pos[i] = s.rs_pos[i - 1];
        s.rs_w[i] = s.rs_w[i - 1];
        s.rs_on[i] = s.rs_on[i - 1];
        --i;
      }
      s.rs_snp[i] = snp;
      s.rs_pos[i] = p;
      s.rs_w[i] = w;
      s.rs_on[i] = 1;
      s.n_rs = n + 1;
    }
    __syncwarp();
  }
  __device__ double rs_total()
  {
    double t = 0;
    for (int i = 0; i < s.n_rs; ++i)
      if (s.rs_on[i]) t += s.rs_w[i];
    return t;
  }
  __device__ uint32_t rs_sample()
  {
    double total = rs_total();
    double r = u01() * total;
    double acc = 0;
    int last = -1;
    for (int i = 0; i < s.n_rs; ++i) {
      if (!s.rs_on[i]) continue;
      last = i;
      acc += s.rs_w[i];
      if (r < acc) return s.rs_snp[i];
    }
    return last >= 0 ? s.rs_snp[last] : 0;
  }

  // ------------------------------------------------------------ moves
  /* src/sampler.hpp:500-515: a new term's missing calls are imputed afresh
     (DataModel::sample_missing_single) before its prior precision is drawn */
  __device__ void prepare_add(uint32_t snp, int type, double* itv, bool missing_draw)
  {
    if (missing_draw && has_miss(snp)) draw_missing(snp);
    if (type == 4) {
      itv[0] = sample_inv_tau2_prior(0);
      itv[1] = sample_inv_tau2_prior(1);
    } else {
      itv[0] = sample_inv_tau2_prior(type);
    }
  }

  // commit the proposed model as the current one (Model::operator=)
  __device__ void accept_model()
  {
    // membership map of the current model: clear old, set new
    int32_t* mi = K.model_inds + (size_t)c * K.p;
    uint32_t* ib = K.inbits + (size_t)c * ((K.p + 31) / 32);
    for (int i = lane; i < cur->k; i += 32) {
      uint32_t sn = cur->loci[i];
      mi[sn] = -1;
      atomicAnd(&ib[sn >> 5], ~(1u << (sn & 31)));
    }
    __syncwarp();
    for (int i = lane; i < nm->k; i += 32) {
      uint32_t sn = nm->loci[i];
      mi[sn] = i;
      atomicOr(&ib[sn >> 5], 1u << (sn & 31));
    }
    __syncwarp();
    copy_model(cur, nm);
  }

  /* src/sampler.hpp:1126-1165 */
  __device__ int prepare_addrem(double& lqf, int ms)
  {
    long long max_adds = (long long)K.p - cur->k, max_rems = cur->k;
    int nrem = 0;
    for (int i = 0; i < ms; ++i) {
      bool add;
      if (max_rems == 0) add = true;
      else if (max_adds == 0) add = false;
      else { lqf += LOG_HALF_D; add = (u01() < 0.5); }
      uint32_t ind;
      if (add) {
        --max_adds;
        double tot = add_total();
        if (K.lrn.on) {
          // mixture of the adaptive proposal and the learned candidates
          const long long wm = s.w_m;
          const double eps = wm > 0 ? K.lrn.mix : 0.0;
          const bool learned = eps > 0 && u01() < eps;
          ind = learned ? mlp_sample(wm) : add_sample();
          double q = (1.0 - eps) * qadd(ind) / tot;
          if (eps > 0) q += eps * (double)mlp_wint(ind) / (double)wm;
          lqf += flog(q);
        } else {
          ind = add_sample();
          lqf += flog(qadd(ind)) - flog(tot);
        }
        add_set_zero(ind, true);
        if (lane == 0) { s.move_isadd[i] = 1; s.move_inds[i] = ind; s.move_map[i] = ind; }
      } else {
        ++nrem;
        --max_rems;
        double tot = rs_total();
        ind = rs_sample();
        lqf += flog(qrem(ind)) - flog(tot);
        rs_set(ind, false);
        if (lane == 0) { s.move_isadd[i] = 0; s.move_inds[i] = ind; s.move_map[i] = -1; }
      }
      __syncwarp();
    }
    return nrem;
  }
  /* src/sampler.hpp:1204-1268 */
  __device__ void do_addrem(double& lqf, double& lqb, double& lmpc, int ms, double* cs, double* sn)
  {
    int last_map = ms - 1;
    for (int i = 0; i < ms; ++i) {
      if (s.move_isadd[i]) continue;
      uint32_t ind = s.move_inds[i];
      add_set_zero(ind, false);
      while (s.move_map[last_map] >= 0) --last_map;
      __syncwarp();
      if (lane == 0) s.move_map[last_map] = ind;
      __syncwarp();
      int mi = find_locus(nm, ind);
      int t_ind = nm->type_inds[mi];
      int type = K.types[t_ind];
      lmpc += lchange_rem(nm->Ns, nm->k, type);
      if (K.n_types > 1) {
        double qa[5], qc[5];
        qtypes(ind, qa, qc);
        lqb += flog(qa[t_ind] / qc[K.n_types - 1]);
      }
      remove_term(nm, mi, cs, sn);
    }
    double itv[2];
    for (int i = 0; i < ms; ++i) {
      if (!s.move_isadd[i]) continue;
      uint32_t ind = s.move_inds[i];
      rs_set(ind, true);
      int t_ind = 0;
      double qa[5], qc[5];
      if (K.n_types > 1) {
        qtypes(ind, qa, qc);
        t_ind = sample_naive(qc, K.n_types);
      }
      int type = K.types[t_ind];
      lmpc += lchange_add(nm->Ns, nm->k, type);
      if (K.n_types > 1) lqf += flog(qa[t_ind] / qc[K.n_types - 1]);
      prepare_add(ind, type, itv, true);
      add_term(nm, ind, t_ind, itv);
    }
  }
  /* src/sampler.hpp:1168-1202 */
  __device__ void backward_prepare_addrem(double& lqb, int ms)
  {
    long long max_adds = (long long)K.p - nm->k, max_rems = nm->k;
    double w_add = add_total(), w_rem = rs_total();
    long long wmb = s.w_m;
    int last_rem = ms - 1;
    for (int i = 0; i < ms; ++i) {
      if (max_adds > 0 && max_rems > 0) lqb += LOG_HALF_D;
      uint32_t ind;
      if (s.move_isadd[i]) {
        --max_rems;
        while (!s.move_isadd[last_rem]) --last_rem;
        ind = (uint32_t)s.move_map[last_rem];
        --last_rem;
        double q = qrem(ind);
        lqb += flog(q) - flog(w_rem);
        w_rem -= q;
      } else {
        --max_adds;
        ind = (uint32_t)s.move_map[i];
        double q = qadd(ind);
        if (K.lrn.on) {
          const double eps = wmb > 0 ? K.lrn.mix : 0.0;
          const long long wi = mlp_wint(ind);
          double qm = (1.0 - eps) * q / w_add;
          if (eps > 0) qm += eps * (double)wi / (double)wmb;
          lqb += flog(qm);
          wmb -= wi;
        } else {
          lqb += flog(q) - flog(w_add);
        }
        w_add -= q;
      }
    }
  }
  /* src/sampler.hpp:899-1123 (delayed rejection off) */
  __device__ int do_addrem_move(double* cs, double* sn)
  {
    int ms = sample_naive(K.q_ms + (size_t)c * 256, K.max_move_size) + 1;
    if (lane == 0) ch->movesize = ms;
    __syncwarp();
    double lqf = 0, lqb = 0, lmpc = 0;
    rs_build_from(cur);
    const int nrem = prepare_addrem(lqf, ms);
    do_addrem(lqf, lqb, lmpc, ms, cs, sn);
    backward_prepare_addrem(lqb, ms);
    double log_r = lqb - lqf;
    log_r += lmpc + nm->ll - cur->ll;
    double* rs = K.r_ms_sum + (size_t)c * 256;
    double* rn = K.r_ms_n + (size_t)c * 256;
    // with delayed rejection the acceptance statistic counts moved SNPs
    // (src/sampler.hpp:1001-1005, 1080)
    const double addv = K.dr ? 0.0 : (log_r >= 0 ? 1.0 : exp(log_r));
    __syncwarp();
    if (lane == 0) { rs[ms - 1] += addv; rn[ms - 1] += 1.0; }
    __syncwarp();
    if (log_r >= 0 || flog(u01()) <= log_r) {
      if (K.dr && lane == 0) rs[ms - 1] += 1.0;
      __syncwarp();
      accept_model();
      return ms;
    }
    if (ms <= (int)K.dr && ms > 1) return delayed_rejection(ms, nrem, cs, sn);
    copy_model(nm, cur);
    for (int i = 0; i < ms; ++i) {
      uint32_t ind = s.move_inds[i];
      if (s.move_isadd[i]) add_set_zero(ind, false);
      else add_set_zero(ind, true);
    }
    return 0;
  }

  /* src/sampler.hpp:1271-1418 */
  __device__ int do_swap_move(double* cs, double* sn)
  {
    long long full = (long long)K.p - cur->k;
    int mm2 = (K.max_move_size + 1) / 2;
    int mms = (int)min((long long)mm2, (full + 1) / 2);
    mms = min(mms, cur->k);
    int ms = sample_naive(K.q_nbs + (size_t)c * 128, mms) + 1;
    if (lane == 0) ch->movesize = ms;
    __syncwarp();
    long long nbh = max(1ll, (full - ms) / 2);
    nbh = min((long long)K.max_nbh, nbh);
    int32_t* cmi = K.model_inds + (size_t)c * K.p;
    const long long p = (long long)K.p;
    for (int im = 0; im < ms; ++im) {
      int mir = (int)floor(u01() * nm->k);
      uint32_t ind_rem = nm->loci[mir];
      long long ind_add;
      int j = 0;
      int mv = (int)floor(u01() * (double)nbh) + 1;
      if (u01() < 0.5) {
        ind_add = ind_rem;
        j = 0;
        while (j < mv) {
          ++ind_add;
          if (ind_add < p) { if (cmi[ind_add] < 0) ++j; }
          else break;
        }
        if (ind_add == p) {
          ind_add = ind_rem;
          mv = mv + mv - j;
          j = 0;
          while (j < mv) {
            --ind_add;
            while (ind_add > 0 && cmi[ind_add] >= 0) --ind_add;
            ++j;
          }
        }
      } else {
        ind_add = ind_rem;
        j = 0;
        if (ind_add > 0) {
          while (j < mv) {
            --ind_add;
            if (ind_add > 0) { if (cmi[ind_add] < 0) ++j; }
            else break;
          }
        }
        if (j < mv) {
          if (cmi[ind_add] < 0) ++j;
          if (j < mv) {
            ind_add = ind_rem;
            mv = mv + mv - j;
            j = 0;
            while (j < mv) {
              ++ind_add;
              while (ind_add < p - 1 && cmi[ind_add] >= 0) ++ind_add;
              ++j;
            }
          }
        }
      }
      int t_ind = nm->type_inds[mir];
      __syncwarp();
      if (lane == 0) {
        s.move_rem[im] = ind_rem;
        s.move_add[im] = (uint32_t)ind_add;
      }
      __syncwarp();
      remove_term(nm, mir, cs, sn);
      __syncwarp();
      if (lane == 0) cmi[ind_add] = t_ind;  // the reference's temporary marking
      __syncwarp();
    }
    double itv[2];
    for (int im = 0; im < ms; ++im) {
      uint32_t ind_add = s.move_add[im];
      int t_ind = (int)(signed char)cmi[ind_add];
      int type = K.types[t_ind];
      prepare_add(ind_add, type, itv, true);
      add_term(nm, ind_add, t_ind, itv);
      __syncwarp();
      if (lane == 0) cmi[ind_add] = -1;
      __syncwarp();
    }
    double log_r = nm->ll - cur->ll;
    if (log_r >= 0 || flog(u01()) <= log_r) {
      accept_model();
      for (int im = 0; im < ms; ++im) {
        add_set_zero(s.move_rem[im], false);
        add_set_zero(s.move_add[im], true);
      }
      return 2 * ms;
    }
    copy_model(nm, cur);
    return 0;
  }

  /* src/sampler.hpp:1421-1669 (delayed rejection off) */
  __device__ int do_statechange_move(double* cs, double* sn)
  {
    long long mms = min((long long)K.max_nbh * 2, min((long long)K.p - 1, (long long)K.max_move_size));
    int ms = sample_naive(K.q_nbc + (size_t)c * 256, (int)mms) + 1;
    if (lane == 0) ch->movesize = ms;
    __syncwarp();
    // the reference takes min(max_nbh, m_g / 2); when 2 nbh + 1 exceeds m_g
    // its wrapped index goes below zero (a size_t out-of-bounds read, UB), so
    // the window is capped at (m_g - 1) / 2 each side, which changes nothing
    // for m_g > 2 max_nbh
    long long nbh = min((long long)K.max_nbh, ((long long)K.p - 1) / 2);
    int mic = (int)floor(u01() * nm->k);
    long long ind_c = nm->loci[mic];
    // the permutation of 2*nbh neighbours is kept in move_map
    for (int i = lane; i < 2 * nbh && i <= BMG_MAX_MS; i += 32) s.move_map[i] = i;
    __syncwarp();
    long long wrap = ind_c + nbh;
    if (ind_c < nbh) wrap += (nbh - ind_c);
    else if (wrap > (long long)K.p - 1) wrap = (long long)K.p - 1;
    for (int im = 0; im < ms; ++im) {
      long long ind = (long long)floor(u01() * (double)(nbh * 2 - im)) + im;
      __syncwarp();
      if (lane == 0) {
        long long t = s.move_map[im];
        s.move_map[im] = s.move_map[ind];
        s.move_map[ind] = t;
      }
      __syncwarp();
    }
    const int32_t* cmi = K.model_inds + (size_t)c * K.p;
    int nadd = 0, nrem = 0;
    for (int im = 0; im < ms; ++im) {
      long long ind = s.move_map[im] + ind_c + 1;
      if (ind > wrap) ind = ind_c - (ind - wrap);
      // nm equals cur here, so cur's membership map answers nm's query
      if (cmi[ind] < 0) { if (lane == 0) s.move_add[nadd] = (uint32_t)ind; ++nadd; }
      else { if (lane == 0) s.move_rem[nrem] = (uint32_t)ind; ++nrem; }
    }
    __syncwarp();
    double lmpc = 0;
    for (int im = 0; im < nrem; ++im) {
      int mir = find_locus(nm, s.move_rem[im]);
      int type = K.types[nm->type_inds[mir]];
      lmpc += lchange_rem(nm->Ns, nm->k, type);
      remove_term(nm, mir, cs, sn);
    }
    double itv[2];
    int t_ind = nm->type_inds[mic];
    int type = K.types[t_ind];
    for (int im = 0; im < nadd; ++im) {
      uint32_t ind_add = s.move_add[im];
      lmpc += lchange_add(nm->Ns, nm->k, type);
      prepare_add(ind_add, type, itv, true);
      add_term(nm, ind_add, t_ind, itv);
    }
    double log_r = lmpc + nm->ll - cur->ll;
    log_r += flog((double)cur->k) - flog((double)nm->k);
    if (log_r >= 0 || flog(u01()) <= log_r) {
      accept_model();
      for (int im = 0; im < nadd; ++im) add_set_zero(s.move_add[im], true);
      for (int im = 0; im < nrem; ++im) add_set_zero(s.move_rem[im], false);
      return ms;
    }
    if (ms <= (int)K.dr && ms > 1) return delayed_rejection_statechange(ms, nadd, nrem, cs, sn);
    copy_model(nm, cur);
    return 0;
  }

  /* src/sampler.hpp:1672-1713 */
  __device__ int do_typeswitch_move(double* cs, double* sn)
  {
    if (lane == 0) ch->movesize = 1;
    __syncwarp();
    int mi = (int)round((cur->k - 1) * u01());
    uint32_t ind = cur->loci[mi];
    int tr = cur->type_inds[mi];
    double qa[5], qc[5], tmp[5];
    qtypes(ind, qa, qc);
    int nt = K.n_types;
    tmp[0] = (tr == 0) ? 0 : qa[0];
    for (int i = 1; i < nt; ++i) tmp[i] = tmp[i - 1] + ((tr == i) ? 0 : qa[i]);
    int ta = sample_naive(tmp, nt);
    int type_add = K.types[ta], type_rem = K.types[tr];
    double itv[2];
    remove_term(nm, mi, cs, sn);
    prepare_add(ind, type_add, itv, false);
    add_term(nm, ind, ta, itv);
    double r = lchange_swi(cur->Ns, type_add, type_rem) + nm->ll - cur->ll -
               flog(qa[ta] / tmp[nt - 1]) + flog(qa[tr] / (qc[nt - 1] - qa[ta]));
    if (r >= 0 || flog(u01()) <= r) {
      accept_model();
      return 1;
    }
    copy_model(nm, cur);
    return 0;
  }

  // ------------------------------------------------- delayed rejection
  // src/sampler.cpp:882-1049 (exhaustive sub-model set, second-stage
  // proposal), src/sampler.hpp:929-1098 and 1547-1618 (the two second stages),
  // src/model.hpp:585-844 (ExhModel), src/symmmatrix.cpp:220-264 (adjacent
  // column swap of a Cholesky factor).  The exhaustive model lives in the
  // chain's slices of K.dr_*; its scalars in shared memory.
  __device__ size_t tri_n() const { return (size_t)km * (km + 1) / 2; }
  __device__ double* drL() const { return K.dr_l + (size_t)c * tri_n(); }
  __device__ double* drV() const { return K.dr_v + (size_t)c * km; }
  __device__ double* drInv() const { return K.dr_inv + (size_t)c * km; }
  __device__ uint8_t* drTi() const { return K.dr_ti + (size_t)c * km; }
  __device__ uint32_t* drX1() const { return K.dr_x1 + (size_t)c * km; }
  __device__ uint32_t* drX2() const { return K.dr_x2 + (size_t)c * km; }
  __device__ double* drPm() const { return K.dr_pm + ((size_t)c << K.dr); }

  /* ExhModel::update_to_model: the proposed model with its first const_loci
     loci fixed; returns its log probability */
  __device__ double dr_update_to_model(int const_loci)
  {
    const DevModel* M = nm;
    {
      const double* ls = Lb(M);
      double* ld = drL();
      const size_t tri = TRI(0, M->llen);
      for (size_t q = lane; q < tri; q += 32) ld[q] = ls[q];
      const double* vs = Vb(M);
      for (int i = lane; i < M->vlen; i += 32) drV()[i] = vs[i];
      for (int i = lane; i < M->xcols; i += 32) drInv()[i] = M->inv[i];
      for (int i = lane; i < M->k; i += 32) {
        drTi()[i] = M->type_inds[i];
        drX1()[i] = M->x_ind1[i];
        drX2()[i] = M->x_ind2[i];
      }
    }
    __syncwarp();
    int vsz = (int)K.m_e;
    if (const_loci > 0) {
      const int ti = drTi()[const_loci - 1];
      vsz = (int)(K.types[ti] == 4 ? drX2()[const_loci - 1] : drX1()[const_loci - 1]) + 1;
    }
    const double* v = drV();
    const double* L0 = drL();
    const double syx = P.nus2_plus_yy - dot(v, v, vsz);
    double a = 0.0, b = 0.0;
    for (int i = lane; i < vsz; i += 32) {
      a += flog(L0[TRI(i, i)]);
      if (i >= 1 && i < (int)K.m_e) b += flog(K.inv_tau2_e[i]);
      else if (i >= (int)K.m_e) b += flog(drInv()[i]);
    }
    const double ldqx = warp_sum_d(a);
    const double ldq = 0.5 * warp_sum_d(b);
    int Ns[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < const_loci; ++i) ++Ns[K.types[drTi()[i]]];
    __syncwarp();
    if (lane == 0) {
      s.dr_ms = const_loci;
      s.dr_vs = vsz;
      s.dr_llen = M->llen;
      s.dr_syx = syx;
      s.dr_ldq = ldq;
      s.dr_ldqx = ldqx;
      s.dr_lmp = 0.0;
      for (int t = 0; t < 5; ++t) s.dr_Ns[t] = Ns[t];
    }
    __syncwarp();
    return ldq - ldqx + P.minus_n_plus_nu_2 * flog(syx);
  }

  /* ExhModel::update_on_add: the next term joins the leading sub-model */
  __device__ double dr_on_add()
  {
    const double* v = drV();
    const double* Lx = drL();
    const int ms = s.dr_ms;
    const int type = K.types[drTi()[ms]];
    int vs = s.dr_vs;
    double syx = s.dr_syx, ldq = s.dr_ldq, ldqx = s.dr_ldqx;
    for (int t = 0; t < (type == 4 ? 2 : 1); ++t) {
      syx -= v[vs] * v[vs];
      ldq += 0.5 * flog(drInv()[vs]);
      ldqx += flog(Lx[TRI(vs, vs)]);
      ++vs;
    }
    int Ns[5];
    for (int t = 0; t < 5; ++t) Ns[t] = s.dr_Ns[t];
    const double lmp = s.dr_lmp + lchange_add(Ns, ms, type);
    __syncwarp();
    if (lane == 0) {
      s.dr_vs = vs;
      s.dr_syx = syx;
      s.dr_ldq = ldq;
      s.dr_ldqx = ldqx;
      s.dr_lmp = lmp;
      s.dr_Ns[type]++;
      s.dr_ms = ms + 1;
    }
    __syncwarp();
    return ldq - ldqx + P.minus_n_plus_nu_2 * flog(syx) + lmp;
  }

  /* SymmMatrix::cholesky_swapadj: columns col and col + 1 trade places, one
     rotation of rows col, col + 1 restores the triangle (and v) */
  __device__ void dr_swapadj(int col)
  {
    double* Lx = drL();
    double* v = drV();
    const double b = Lx[TRI(col + 1, col + 1)];
    __syncwarp();
    for (int r = lane; r <= col; r += 32) {
      const double x = Lx[TRI(r, col)], y = Lx[TRI(r, col + 1)];
      Lx[TRI(r, col)] = y;
      Lx[TRI(r, col + 1)] = x;
    }
    __syncwarp();
    if (lane == 0) Lx[TRI(col + 1, col + 1)] = 0.0;
    __syncwarp();
    const double a = Lx[TRI(col, col)];
    // drotg(a, b) with r taking the sign of the larger input, then the
    // reference's flip to a positive diagonal
    double rv = 0.0, cc = 1.0, ss = 0.0;
    const double h2 = a * a + b * b;
    if (h2 > 0.0) {
      const double sgn = (fabs(a) > fabs(b) ? a : b) < 0.0 ? -1.0 : 1.0;
      const double ri = rsqrt(h2) * sgn;
      rv = h2 * ri;
      cc = a * ri;
      ss = b * ri;
    }
    if (rv < 0.0) {
      rv = -rv;
      ss = -ss;
      cc = -cc;
    }
    const int llen = s.dr_llen;
    for (int i = col + 1 + lane; i < llen; i += 32) {
      const double x = Lx[TRI(col, i)], y = Lx[TRI(col + 1, i)];
      Lx[TRI(col, i)] = y * ss + x * cc;
      Lx[TRI(col + 1, i)] = x * ss - y * cc;
    }
    if (lane == 0) {
      Lx[TRI(col, col)] = rv;
      const double x = v[col], y = v[col + 1];
      v[col] = y * ss + x * cc;
      v[col + 1] = x * ss - y * cc;
    }
    __syncwarp();
  }
  __device__ void dr_swap_inv(uint32_t a, uint32_t b)
  {
    if (lane == 0) {
      double* iv = drInv();
      const double t = iv[a];
      iv[a] = iv[b];
      iv[b] = t;
    }
    __syncwarp();
  }

  /* ExhModel::update_on_moveleft: the last term of the leading sub-model
     trades places with the one before it, which leaves the sub-model */
  __device__ double dr_on_moveleft()
  {
    const double* v = drV();
    int ms = s.dr_ms - 1;
    const int ind_keep = ms, ind_rem = ms - 1;
    uint8_t* ti = drTi();
    uint32_t* x1 = drX1();
    uint32_t* x2 = drX2();
    const int type_keep = K.types[ti[ind_keep]], type_rem = K.types[ti[ind_rem]];
    int vs = s.dr_vs;
    double syx = s.dr_syx, ldq = s.dr_ldq, ldqx = s.dr_ldqx;
    {
      const double* Lx = drL();
      --vs;
      syx += v[vs] * v[vs];
      ldqx -= flog(Lx[TRI(vs, vs)]);
      if (type_keep == 4) {
        --vs;
        syx += v[vs] * v[vs];
        ldqx -= flog(Lx[TRI(vs, vs)]);
      }
      --vs;
      syx += v[vs] * v[vs];
      ldq -= 0.5 * flog(drInv()[vs]);
      ldqx -= flog(Lx[TRI(vs, vs)]);
      if (type_rem == 4) {
        --vs;
        syx += v[vs] * v[vs];
        ldq -= 0.5 * flog(drInv()[vs]);
        ldqx -= flog(Lx[TRI(vs, vs)]);
      }
    }
    __syncwarp();
    if (lane == 0) {
      const uint8_t t = ti[ind_keep];
      ti[ind_keep] = ti[ind_rem];
      ti[ind_rem] = t;
    }
    __syncwarp();
    const uint32_t k1 = x1[ind_keep], k2 = x2[ind_keep], r1 = x1[ind_rem], r2 = x2[ind_rem];
    if (type_rem == 4) {
      if (type_keep == 4) {
        int si = (int)r2;
        dr_swapadj(si);
        ++si;
        dr_swapadj(si);
        si -= 2;
        dr_swapadj(si);
        ++si;
        dr_swapadj(si);
        dr_swap_inv(k1, r2);
        dr_swap_inv(k1, k2);
        dr_swap_inv(r1, r2);
        dr_swap_inv(k1, r2);
      } else {
        int si = (int)r2;
        dr_swapadj(si);
        --si;
        dr_swapadj(si);
        dr_swap_inv(r2, k1);
        dr_swap_inv(r1, r2);
        if (lane == 0) {
          x2[ind_keep] = k1;
          x1[ind_keep] = k1 - 1;
        }
      }
    } else {
      if (type_keep == 4) {
        int si = (int)r1;
        dr_swapadj(si);
        ++si;
        dr_swapadj(si);
        dr_swap_inv(r1, k1);
        dr_swap_inv(k1, k2);
        if (lane == 0) {
          x2[ind_rem] = k1;
          x1[ind_keep] = k2;
        }
      } else {
        dr_swapadj((int)r1);
        dr_swap_inv(k1, r1);
      }
    }
    __syncwarp();
    {
      const double* Lx = drL();
      syx -= v[vs] * v[vs];
      ldqx += flog(Lx[TRI(vs, vs)]);
      ++vs;
      if (type_keep == 4) {
        syx -= v[vs] * v[vs];
        ldqx += flog(Lx[TRI(vs, vs)]);
        ++vs;
      }
    }
    int Ns[5];
    for (int t = 0; t < 5; ++t) Ns[t] = s.dr_Ns[t];
    const double lmp = s.dr_lmp + lchange_rem(Ns, ms + 1, type_rem);
    __syncwarp();
    if (lane == 0) {
      s.dr_ms = ms;
      s.dr_vs = vs;
      s.dr_syx = syx;
      s.dr_ldq = ldq;
      s.dr_ldqx = ldqx;
      s.dr_lmp = lmp;
      s.dr_Ns[type_rem]--;
    }
    __syncwarp();
    return ldq - ldqx + P.minus_n_plus_nu_2 * flog(syx) + lmp;
  }

  __device__ void dr_put(double* pm, unsigned idx, double v, double& mx)
  {
    if (lane == 0) pm[idx] = v;
    if (v > mx) mx = v;
  }

  /* compute_exhaustive_modelset (src/sampler.cpp:882-978): the log
     probability of each of the 2^n sub-models of the last n terms, bit i of
     the index = term i of the block in the model */
  __device__ double dr_exhaustive(int n_inds, double* pm)
  {
    int ci[BMG_DR_MAX];
    for (int i = 0; i < n_inds; ++i) ci[i] = i;
    unsigned cb = 0;
    int msz = 0;
    double mx = -INFINITY;
    dr_put(pm, 0, dr_update_to_model(s.dr_ms), mx);
    for (int i = 0; i < n_inds; ++i) {
      ++msz;
      if (i > 1) {
        ++msz;
        dr_on_add();
      }
      cb = (1u << msz) - 1;
      dr_put(pm, cb, dr_on_add(), mx);
      for (int j = 0; j < i; ++j) {
        --msz;
        const int t = ci[msz - 1];
        ci[msz - 1] = ci[msz];
        ci[msz] = t;
        cb &= ~(1u << t);
        dr_put(pm, cb, dr_on_moveleft(), mx);
      }
      const unsigned nmodels = (1u << i) - i - 1;
      unsigned jj = 0, nK = 0;
      int do_lefts = 0;
      while (jj < nmodels) {
        if (do_lefts < 2) {
          ++msz;
          const int t = ci[msz];
          ci[msz] = ci[msz - 1];
          ci[msz - 1] = t;
          cb |= (1u << t);
          dr_on_add();
          dr_on_add();
          dr_put(pm, cb, dr_on_moveleft(), mx);
          ++jj;
          ++do_lefts;
        } else {
          ++nK;
          int Kb = 0;
          while (((nK >> Kb) & 1u) == 0) ++Kb;
          for (int k2 = 0; k2 <= Kb; ++k2) {
            --msz;
            const int t = ci[msz - 1];
            ci[msz - 1] = ci[msz];
            ci[msz] = t;
            cb &= ~(1u << t);
            dr_put(pm, cb, dr_on_moveleft(), mx);
            ++jj;
          }
          do_lefts = 0;
        }
      }
    }
    __syncwarp();
    return mx;
  }

  /* compute_proposal_probs_for_exh_modelset (src/sampler.cpp:980-1049): the
     log probability of proposing each sub-model from the model without the
     block's terms (adds in order, removals in reverse), one sub-model per
     lane at a time */
  __device__ void dr_proposal_probs(int n_inds, double z_add, double z_rem, long long const_loci, double* pm)
  {
    const unsigned nmodels = 1u << n_inds;
    const bool use_types = K.n_types > 1;
    for (unsigned i = lane; i < nmodels; i += 32) {
      long long max_adds = (long long)K.p - const_loci, max_rems = const_loci;
      double z_a = z_add, z_r = z_rem;
      unsigned isadd = 0;
      for (int j = 0; j < n_inds; ++j) {
        const int nind = s.dr_b2o[j];
        if ((i >> j) & 1u) {
          z_a -= s.dr_qa[nind];
          z_r += s.dr_qr[nind];
          ++max_rems;
          --max_adds;
        } else {
          isadd |= 1u << nind;
        }
      }
      double lp = 0.0;
      int last_rem = n_inds - 1;
      for (int j = 0; j < n_inds; ++j) {
        if (max_adds > 0 && max_rems > 0) lp += LOG_HALF_D;
        if ((isadd >> j) & 1u) {
          --max_adds;
          lp += flog(s.dr_qa[j]) - flog(z_a);
          z_a -= s.dr_qa[j];
          if (use_types) lp += s.dr_lqt[j];
        } else {
          --max_rems;
          while ((isadd >> last_rem) & 1u) --last_rem;
          lp += flog(s.dr_qr[last_rem]) - flog(z_r);
          z_r -= s.dr_qr[last_rem];
          --last_rem;
        }
      }
      pm[i] += lp;
    }
    __syncwarp();
  }

  /* src/sampler.hpp:1009-1028: each sub-model below 2^(n-1) is paired with
     its complement; the pair's weight (the difference of their
     probabilities) goes to the likelier one.  A pair is drawn by its
     cumulative weight (one uniform, src/utils.cpp:73-101) and the sub-model
     carrying it is returned. */
  __device__ unsigned dr_sample_pair(int n, double mx, double* pm)
  {
    const unsigned nmodels = 1u << n, mask = nmodels - 1, half = nmodels >> 1;
    double carry = 0.0;
    for (unsigned base = 0; base < half; base += 32) {
      const unsigned i = base + lane;
      double w = 0.0;
      if (i < half) {
        const unsigned j = (~i) & mask;
        const double a = pm[j] - pm[i];
        if (a > 0) {
          w = exp(pm[j] - mx) * (1 - exp(-a));
          pm[j] = -1.0;
        } else {
          w = exp(pm[i] - mx) * (1 - exp(a));
          pm[j] = 1.0;
        }
      }
      // inclusive prefix within the chunk, then the running total
      for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(FULL_MASK, w, o);
        if (lane >= o) w += t;
      }
      w += carry;
      if (i < half) pm[i] = w;
      carry = __shfl_sync(FULL_MASK, w, 31);
    }
    __syncwarp();
    const double rr = u01() * pm[half - 1];
    unsigned pick = half - 1;
    for (unsigned base = 0; base < half; base += 32) {
      const unsigned i = base + lane;
      const unsigned hit = __ballot_sync(FULL_MASK, i < half && rr < pm[i]);
      if (hit) {
        pick = base + __ffs(hit) - 1;
        break;
      }
    }
    const unsigned comp = (~pick) & mask;
    if (pm[comp] < 0) pick = comp;
    __syncwarp();
    return pick;
  }

  // re-add a SNP of the current model to nm with the current model's precision
  __device__ void dr_readd(uint32_t ind)
  {
    const int cmi = K.model_inds[(size_t)c * K.p + ind];
    const int t_ind = cur->type_inds[cmi];
    double itv[2];
    itv[0] = cur->inv[cur->x_ind1[cmi]];
    itv[1] = (K.types[t_ind] == 4) ? cur->inv[cur->x_ind2[cmi]] : 0.0;
    add_term(nm, ind, t_ind, itv);
  }
  // keep the sub-model `sampled` of nm's last n terms: drop the others
  __device__ void dr_keep(unsigned sampled, int n, int const_loci, double* cs, double* sn)
  {
    unsigned rem = sampled;
    for (int i = 0; i < n; ++i) {
      if ((rem & 1u) == 0) {
        remove_term(nm, const_loci + i, cs, sn);
        --const_loci;
      }
      rem >>= 1;
    }
  }

  /* src/sampler.hpp:929-1098: the second stage after a rejected multi-SNP
     add/remove move */
  __device__ int delayed_rejection(int ms, int ms_rem, double* cs, double* sn)
  {
    const int const_loci = cur->k - ms_rem;
    const int ms_add = ms - ms_rem;
    double z_add = add_total(), z_rem = rs_total();
    const unsigned newmodel = (1u << ms_add) - 1;
    for (int i = 0; i < ms; ++i) {
      const uint32_t ind = s.move_inds[i];
      if (s.move_isadd[i]) {
        z_add += qadd(ind);
        z_rem -= qrem(ind);
      } else {
        dr_readd(ind);
      }
    }
    for (int i = 0; i < ms; ++i) {
      const uint32_t ind = (uint32_t)s.move_map[i];
      const int mi = find_locus(nm, ind);
      double lqt = 0.0;
      if (K.n_types > 1) {
        double qa[5], qc[5];
        qtypes(ind, qa, qc);
        lqt = flog(qa[nm->type_inds[mi]] / qc[K.n_types - 1]);
      }
      const double qa1 = qadd(ind), qr1 = qrem(ind);
      __syncwarp();
      if (lane == 0) {
        s.dr_b2o[mi - const_loci] = i;
        s.dr_qa[i] = qa1;
        s.dr_qr[i] = qr1;
        s.dr_lqt[i] = lqt;
      }
      __syncwarp();
    }
    double* pm = drPm();
    if (lane == 0) s.dr_ms = const_loci;
    __syncwarp();
    const double mx = dr_exhaustive(ms, pm);
    dr_proposal_probs(ms, z_add, z_rem, const_loci, pm);
    const unsigned mask = (1u << ms) - 1;
    const unsigned sampled = dr_sample_pair(ms, mx, pm);
    if (sampled == ((~newmodel) & mask)) {
      copy_model(nm, cur);
      for (int i = 0; i < ms; ++i) {
        const uint32_t ind = s.move_inds[i];
        add_set_zero(ind, !s.move_isadd[i]);
      }
      return 0;
    }
    int moved = 0;
    for (int i = 0; i < ms; ++i) {
      const bool in_new = (newmodel >> i) & 1u;
      const uint32_t ind = (uint32_t)s.move_map[s.dr_b2o[i]];
      if ((sampled >> i) & 1u) {
        if (!in_new) add_set_zero(ind, true);
        else ++moved;
      } else {
        if (in_new) add_set_zero(ind, false);
        else ++moved;
      }
    }
    dr_keep(sampled, ms, const_loci, cs, sn);
    double* rsum = K.r_ms_sum + (size_t)c * 256;
    __syncwarp();
    if (lane == 0) rsum[ms - 1] += (double)moved / (double)ms;
    __syncwarp();
    accept_model();
    return moved;
  }

  /* src/sampler.hpp:1547-1618: the second stage after a rejected state
     change; each sub-model's probability includes the choice of the central
     SNP among its loci */
  __device__ int delayed_rejection_statechange(int ms, int ms_add, int ms_rem, double* cs, double* sn)
  {
    const int const_loci = cur->k - ms_rem;
    const unsigned newmodel = (1u << ms_add) - 1;
    for (int i = 0; i < ms_rem; ++i) dr_readd(s.move_rem[i]);
    double* pm = drPm();
    if (lane == 0) s.dr_ms = const_loci;
    __syncwarp();
    const double mx = dr_exhaustive(ms, pm);
    const unsigned nmodels = 1u << ms, mask = nmodels - 1;
    for (unsigned i = lane; i < nmodels; i += 32) pm[i] -= flog((double)(const_loci + __popc(i)));
    __syncwarp();
    const unsigned sampled = dr_sample_pair(ms, mx, pm);
    if (sampled == ((~newmodel) & mask)) {
      copy_model(nm, cur);
      return 0;
    }
    int moved = 0;
    for (int i = 0; i < ms; ++i) {
      const bool in_new = (newmodel >> i) & 1u;
      if ((sampled >> i) & 1u) {
        if (in_new) {
          ++moved;
          add_set_zero(s.move_add[i], true);
        }
      } else if (!in_new) {
        ++moved;
        add_set_zero(s.move_rem[i - ms_add], false);
      }
    }
    dr_keep(sampled, ms, const_loci, cs, sn);
    accept_model();
    return moved;
  }

  /* src/sampler.hpp:1715-1769 */
  __device__ void adapt_move_size()
  {
    double* q_p0 = K.q_p0_ms + (size_t)c * 256;
    const double* rs = K.r_ms_sum + (size_t)c * 256;
    const double* rn = K.r_ms_n + (size_t)c * 256;
    int mx = K.max_move_size;
    double pms = ch->p_move_size;
    if (K.acpt_goal > 0) {
      double t = fmax(1.0, ch->k_move_size * (double)ch->p_proposal_n);
      double ar = (double)ch->n_acpt[0] / (double)ch->n_moves[0];
      pms = pms + (K.acpt_goal - ar) / (2.0 + t);
      pms = fmax(fmin(pms, 0.99), 0.01);
      if (lane == 0) { ch->n_acpt[0] = 1; ch->n_moves[0] = 2; }
    } else {
      // Evaluated without FMA contraction, with pow() from the host table, so
      // that equal inputs give the reference's rounding: when one move size
      // has data the criterion is flat in p and rounding picks the grid point.
      double q = 1 - pms;
      double pw = K.ms_pow[50];
      for (int j = 0; j < 50; ++j)
        if (K.ms_grid[j] == pms) { pw = K.ms_pow[j]; break; }
      if (pms != K.ms_init && pw == K.ms_pow[50]) {
        bool found = false;
        for (int j = 0; j < 50; ++j) found = found || (K.ms_grid[j] == pms);
        if (!found) pw = pow(q, (double)mx);
      }
      double zp = 1 - pw;
      double q_p = pms / zp;
      for (int i = 0; i < mx; ++i) {
        double nv = __dadd_rn(q_p0[i], q_p);
        __syncwarp();
        if (lane == 0) q_p0[i] = nv;
        q_p = __dmul_rn(q_p, q);
      }
      __syncwarp();
      // grid point j = lane, lane + 32 (the host table holds the grid's
      // sequentially accumulated values); the first strict maximum wins, as
      // in the reference's ascending loop, and 0.01 when none is finite
      double hb = -INFINITY;
      int jb = 1 << 30;
      for (int j = lane; j < 50; j += 32) {
        const double pp = K.ms_grid[j];
        double h = 0.0, z = 0.0, qq = 1.0 - pp, qp = pp;
        for (int i = 0; i < mx; ++i) {
          double ratio = __ddiv_rn(qp, q_p0[i]);
          h = __dadd_rn(h, __dmul_rn(__dmul_rn((double)(i + 1), rs[i]), ratio));
          z = __dadd_rn(z, __dmul_rn(rn[i], ratio));
          qp = __dmul_rn(qp, qq);
        }
        h = __ddiv_rn(h, z);
        if (h > hb) { hb = h; jb = j; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ho = __shfl_xor_sync(FULL_MASK, hb, o);
        const int jo = __shfl_xor_sync(FULL_MASK, jb, o);
        if (ho > hb || (ho == hb && jo < jb)) { hb = ho; jb = jo; }
      }
      pms = (hb > -INFINITY) ? K.ms_grid[jb] : 0.01;
    }
    // Utils::geometric_dist_cdf
    double* qms = K.q_ms + (size_t)c * 256;
    double q = 1 - pms, qp = q;
    for (int i = lane; i < mx; i += 32) {
      double qi = q;
      for (int t = 0; t < i; ++t) qi *= qp;
      qms[i] = 1 - qi;
    }
    if (lane == 0) ch->p_move_size = pms;
    __syncwarp();
  }
};

// ------------------------------------------------------------ bulk phases
// All 256 threads: fitted values of the current model's genotype columns in
// fixed point (coefficients round(beta * 2^s)), the covariate part in FP64,
// and the requested sums; optionally the residual limbs for the scan.
#define BULK_PVE 1
#define BULK_ALPHA 2
#define BULK_RESID 4
#define BULK_YHAT 8   // with BULK_RESID: the residual is y - K.yhat, the fitted values given

// a 128-bit integer as the nearest-ish double (two roundings: relative error
// below 2^-52)
__device__ __forceinline__ double i128_to_double(__int128 v)
{
  const bool neg = v < 0;
  const unsigned __int128 u = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
  const double d = (double)(unsigned long long)(u >> 64) * 18446744073709551616.0 + (double)(unsigned long long)u;
  return neg ? -d : d;
}

__device__ void bulk_phase(const DevConst& K, int c, MoveShared& s, BulkCols& bc)
{
  const DevPheno& P = s.phs;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int mode = s.bulk_mode, nt = s.bulk_nterm, sh = s.bulk_s;
  const int me = K.m_e;
  const double sc = ldexp(1.0, -sh);
  double s1g = 0, s2g = 0, s1e = 0, s2e = 0, s1t = 0, s2t = 0, ymax = 0;
  long long rsum = 0;
  const uint32_t L = K.limbs_n;
  // Model::compute_pve (src/model.hpp:359-371) leaves y_hat untouched before
  // adding E beta_E when the model has no genotype term and there are
  // covariates, so y_hat then accumulates; the scan reads that y_hat
  // (src/sampler.cpp:735).  The same update is reproduced here.
  const bool stale = (mode & BULK_YHAT) || ((nt == 0) && (me > 1));
  // Without covariates the PVE pass needs only sum x'b and sum (x'b)^2 over
  // the sample (the covariate part is the constant), and nothing reads y_hat
  // back: both sums are taken exactly in 128-bit integers from the
  // fixed-point fitted values, with no FP64 instruction per individual.
  const bool ifast = (me <= 1) && (mode & BULK_PVE) && !(mode & (BULK_YHAT | BULK_ALPHA));
  __int128 ia = 0, ia2 = 0;
  double* yhat = K.yhat + (size_t)c * K.n;
  const int dsh = P.sy - sh;
  // the model's missing calls at their imputed values: the codes give 0
  // there, so coef x_t(value) goes into a per-individual correction first
  long long* mfit = K.miss_total ? K.miss_fit + (size_t)c * K.n_pad : nullptr;
  if (mfit && nt > 0) {
    for (int j = 0; j < nt; ++j) {
      const uint32_t sj = bc.snp[j];
      const long long o0 = K.miss_off[sj], o1 = K.miss_off[sj + 1];
      const long long cf = bc.coef[j];
      const int t = bc.term[j];
      for (long long q = o0 + tid; q < o1; q += nth) {
        const long long add = cf * gval_term(K.miss_val[(size_t)c * K.miss_total + q], t);
        if (add) atomicAdd(reinterpret_cast<unsigned long long*>(&mfit[K.miss_ind[q]]), (unsigned long long)add);
      }
    }
    __syncthreads();
  }
  // a thread takes 16 individuals at a time: one 32-bit word of every model
  // column's packed codes, so each column costs one coalesced load per word
  const uint32_t words = (uint32_t)(K.n_pad / 16);
  for (uint32_t w = tid; w < words; w += nth) {
    long long yg16[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) yg16[q] = 0;
    if ((uint64_t)16 * w < K.n) {
      for (int j = 0; j < nt; ++j) {
        const uint32_t code = reinterpret_cast<const uint32_t*>(K.geno + (size_t)bc.snp[j] * K.gs)[w];
        const int t = bc.term[j];
        const long long vh = coefH(t) * bc.coef[j], vr = coefR(t) * bc.coef[j];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const uint32_t c2 = (code >> (2 * q)) & 3u;  // 2 = het, 3 = hom-alt
          yg16[q] += (c2 == 2u) ? vh : ((c2 == 3u) ? vr : 0ll);
        }
      }
      if (mfit) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const uint64_t i = (uint64_t)16 * w + q;
          if (i < K.n) {
            const long long f = mfit[i];
            if (f) {
              yg16[q] += f;
              mfit[i] = 0;
            }
          }
        }
      }
    }
    long long R16[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const uint64_t i = (uint64_t)16 * w + q;
      // individuals outside the chain's sample have no residual
      const bool live = i < K.n && (!P.mask2 || ((P.mask2[i >> 5] >> (2 * (i & 31))) & 1ull));
      const long long yg = yg16[q];
      double ye = 0;
      if (ifast) {
        if (live) {
          ia += yg;
          ia2 += (__int128)yg * yg;
        }
      } else if (live) {
        if (me > 1) {
          for (int e = 0; e < me; ++e) ye += K.e[(size_t)e * K.n + i] * s.bulk_e[e];
        } else {
          ye = s.bulk_b0;
        }
      }
      const double ygd = ifast ? 0.0 : (double)yg * sc;
      double yh = 0;
      if (!ifast && live && (mode & BULK_PVE)) {
        yh = stale ? yhat[i] + ye : ygd + ye;
        yhat[i] = yh;
        ymax = fmax(ymax, fabs(yh));
      }
      if (!ifast && live && (mode & (BULK_PVE | BULK_ALPHA))) {
        s1g += ygd;
        s2g += ygd * ygd;
        if (mode & BULK_ALPHA) {
          // eb = E beta_E - y, xb = fitted genotype part
          s1e += (ye - P.y[i]) * ygd;
        } else {
          s1e += ye;
          s2e += ye * ye;
          const double yt = ygd + ye;
          s1t += yt;
          s2t += yt * yt;
        }
      }
      long long R = 0;
      if (live && (mode & BULK_RESID)) {
        const long long Y = P.yint[i];
        const long long Ys = (dsh > 0) ? ((Y + (1ll << (dsh - 1))) >> dsh) : (Y << (-dsh));
        if (stale) {
          const double yv = (mode & BULK_PVE) ? yh : yhat[i];
          R = Ys - __double2ll_rn(yv * ldexp(1.0, sh));
        } else {
          const long long E = (me > 1) ? __double2ll_rn(ye * ldexp(1.0, sh)) : s.bulk_b0i;
          R = Ys - E - yg;
        }
        K.resid[(size_t)c * K.n_pad + i] = R;
      }
      R16[q] = R;
      rsum += R;
    }
    if (mode & BULK_RESID) {
      // balanced base-256 digits of the 16 residuals, exact as bf16, stored
      // as two 16-byte vectors per digit
      for (uint32_t l = 0; l < L; ++l) {
        uint32_t pk[8];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int d8 = (int)(signed char)(R16[q] & 0xff);
          R16[q] = (R16[q] - d8) >> 8;
          const uint32_t bits = __float_as_uint((float)d8) >> 16;
          if (q & 1) pk[q >> 1] |= bits << 16;
          else pk[q >> 1] = bits;
        }
        uint4* dst = reinterpret_cast<uint4*>(K.limbs + ((size_t)c * L + l) * K.n_pad + (size_t)16 * w);
        dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
      }
    }
  }
  // block reduction
  const int w = tid >> 5, ln = tid & 31;
  if (ifast) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long a0 = __shfl_xor_sync(FULL_MASK, (unsigned long long)ia, o);
      const unsigned long long a1 = __shfl_xor_sync(FULL_MASK, (unsigned long long)(ia >> 64), o);
      const unsigned long long b0 = __shfl_xor_sync(FULL_MASK, (unsigned long long)ia2, o);
      const unsigned long long b1 = __shfl_xor_sync(FULL_MASK, (unsigned long long)(ia2 >> 64), o);
      ia += (__int128)(((unsigned __int128)a1 << 64) | a0);
      ia2 += (__int128)(((unsigned __int128)b1 << 64) | b0);
    }
    if (ln == 0) {
      s.bi[w][0] = (unsigned long long)ia;
      s.bi[w][1] = (unsigned long long)(ia >> 64);
      s.bi[w][2] = (unsigned long long)ia2;
      s.bi[w][3] = (unsigned long long)(ia2 >> 64);
    }
  } else {
    double v6[6] = {s1g, s2g, s1e, s2e, s1t, s2t};
    for (int q = 0; q < 6; ++q) {
      double r = warp_sum_d(v6[q]);
      if (ln == 0) s.bd[w][q] = r;
    }
    for (int o = 16; o > 0; o >>= 1) ymax = fmax(ymax, __shfl_xor_sync(FULL_MASK, ymax, o));
    if (ln == 0) s.bmax[w] = ymax;
  }
  long long rs = warp_sum_ll(rsum);
  if (ln == 0) s.bl[w][0] = rs;
  __syncthreads();
  if (tid == 0) {
    if (ifast) {
      __int128 ta = 0, tb = 0;
      for (int ww = 0; ww < (nth >> 5); ++ww) {
        ta += (__int128)(((unsigned __int128)s.bi[ww][1] << 64) | s.bi[ww][0]);
        tb += (__int128)(((unsigned __int128)s.bi[ww][3] << 64) | s.bi[ww][2]);
      }
      // sum x'b and sum (x'b)^2 at the scales 2^-sh and 2^-2sh; the
      // covariate part is the constant b0 on each of the sample's n
      const double s1 = i128_to_double(ta) * sc, s2 = i128_to_double(tb) * (sc * sc);
      const double b0 = s.bulk_b0, nn = P.n;
      s.bsum[0] = s1;
      s.bsum[1] = s2;
      s.bsum[2] = nn * b0;
      s.bsum[3] = nn * b0 * b0;
      s.bsum[4] = s1 + nn * b0;
      s.bsum[5] = s2 + 2.0 * b0 * s1 + nn * b0 * b0;
      s.bmax[0] = 0.0;
    } else {
      for (int q = 0; q < 6; ++q) {
        double t = 0;
        for (int ww = 0; ww < (nth >> 5); ++ww) t += s.bd[ww][q];
        s.bsum[q] = t;
      }
    }
    long long t = 0;
    for (int ww = 0; ww < (nth >> 5); ++ww) t += s.bl[ww][0];
    s.bsuml[0] = t;
    if ((mode & BULK_PVE) && !ifast) {
      double m = 0;
      for (int ww = 0; ww < (nth >> 5); ++ww) m = fmax(m, s.bmax[ww]);
      s.chs.yhat_absmax = m;
    }
  }
  __syncthreads();
}

// warp 0: fill the bulk column list and coefficients from the current model
__device__ void bulk_setup(Warp& W, BulkCols& bc, int mode)
{
  DevModel* M = W.cur;
  const DevConst& K = W.K;
  int me = K.m_e, bl = M->blen, xc = M->xcols;
  int nt = min(bl, xc) - me;
  if (nt < 0 || (mode & BULK_YHAT)) nt = 0;
  double bound = 0;
  for (int j = 0; j < nt; ++j) bound += 2.0 * fabs(M->beta[me + j]);
  int sh;
  if (mode & BULK_RESID) {
    // |r_i| <= max|y| + sum_e max|E_e| |beta_e| + sum_j 2 |beta_j|; the limbs
    // hold |R| < 2^(8L-1)
    double eb = 0;
    for (int e = 0; e < me && e < bl; ++e) eb += K.e_absmax[e] * fabs(M->beta[e]);
    double tot = bound + W.P.y_absmax + eb + 1e-300;
    if (mode & BULK_YHAT) tot = W.P.y_absmax + W.s.yhat_given_max + 1e-300;
    else if (nt == 0 && me > 1) tot += W.ch->yhat_absmax;  // the accumulated y_hat
    int e2 = (int)ceil(log2(tot));
    // the limbs hold |R| < 2^(8L-1); the scan's exact int64 sums of n
    // products |x R| <= 2 |R| need |R| < 2^(61 - log2 n) as well
    const int lgn = 64 - __clzll((long long)(K.n > 1 ? K.n - 1 : 1));
    sh = min((int)(8 * K.limbs_n - 3), 61 - lgn) - e2;
  } else {
    // fitted genotype values stay below 2^52 so they convert to double exactly
    int e2 = (int)ceil(log2(bound + 1e-300));
    sh = 51 - e2;
  }
  if (sh > 60) sh = 60;
  double scl = ldexp(1.0, sh);
  for (int j = W.lane; j < nt; j += 32) {
    bc.snp[j] = M->xc_snp[me + j];
    bc.term[j] = (int8_t)M->xc_type[me + j];
    bc.coef[j] = __double2ll_rn(M->beta[me + j] * scl);
  }
  if (W.lane == 0) {
    W.s.bulk_mode = mode;
    W.s.bulk_nterm = nt;
    W.s.bulk_s = sh;
    W.s.bulk_b0 = (bl > 0) ? M->beta[0] : 0.0;
    W.s.bulk_b0i = __double2ll_rn(W.s.bulk_b0 * scl);
    for (int e = 0; e <= BMG_MAX_COV; ++e) W.s.bulk_e[e] = (e < me && e < bl) ? M->beta[e] : 0.0;
  }
  __syncwarp();
}

// ------------------------------------------------------------- RB step
/* src/sampler.cpp:731-811: everything of an RB step except the p-wide scan.
   With scan_only the flags ask for p_r only and no counter moves. */
__device__ void prep_rb(Warp& W, bool scan_only)
{
  const DevConst& K = W.K;
  DevChain* ch = W.ch;
  RbParams* rp = K.rb + W.c;
  DevModel* M = W.cur;
  bool do_scan, adapt;
  int acc_rao = 0;
  double rz1 = 0, rz2 = 0, pz1 = 0, pz2 = 0;
  if (scan_only) {
    do_scan = true;
    adapt = false;
  } else {
    do_scan = !K.flat_proposal_dist || ch->n_rao_burnin == 0;
    if (ch->n_rao_burnin == 0) {
      rz1 = (double)(ch->p_rao_n + 1);
      rz2 = (double)ch->p_rao_n / rz1;
      acc_rao = 1;
    }
    uint64_t burn = ch->n_rao_burnin;
    if (burn > 0) burn--;
    adapt = K.adaptation || burn > 0;
    pz1 = (double)(ch->p_proposal_n + 1);
    pz2 = (double)ch->p_proposal_n / pz1;
    __syncwarp();
    if (W.lane == 0) {
      if (acc_rao) ch->p_rao_n++;
      ch->n_rao_burnin = burn;
    }
  }
  // the missing calls outside the model are imputed before the scan
  // (src/sampler.cpp:731-736, DataModel::sample_missing): one slot per call
  // in SNP and call order, the model's SNPs skipped.  The model's SNPs go to
  // K.miss_inm ascending, with the missing calls of the listed SNPs before
  // each, so that the scan's imputation finds every call's slot.
  if (do_scan && K.miss_total) {
    long long* inm = K.miss_inm + (size_t)W.c * 2 * K.km;
    const int k = M->k;
    for (int i = W.lane; i < k; i += 32) {
      const uint32_t si = M->loci[i];
      int rank = 0;
      for (int q = 0; q < k; ++q) rank += M->loci[q] < si;
      inm[rank] = si;
    }
    __syncwarp();
    long long tot_in = 0;
    if (W.lane == 0) {
      for (int q = 0; q < k; ++q) {
        inm[K.km + q] = tot_in;
        const uint32_t sq = (uint32_t)inm[q];
        tot_in += K.miss_off[sq + 1] - K.miss_off[sq];
      }
      inm[K.km + k] = tot_in;
      rp->miss_slot = W.rng.slot;
      rp->n_inm = k;
    }
    tot_in = __shfl_sync(FULL_MASK, tot_in, 0);
    W.rng.slot += K.miss_total - (uint64_t)tot_in;
    __syncwarp();
  }
  // per-SNP tau2 draws of the scan (src/sampler.cpp:99-106) take p * terms
  // consecutive slots, one per (SNP, allowed term) in the reference's order
  uint64_t slot0 = W.rng.slot;
  if (do_scan && K.use_individual_tau2) W.rng.slot += K.p * (uint64_t)K.n_terms;
  if (W.lane == 0) {
    rp->alpha2 = ch->alpha2;
    rp->rng_slot = slot0;
    rp->key0 = W.rng.key0;
    rp->key1 = W.rng.key1;
    rp->do_scan = do_scan;
    rp->acc_rao = acc_rao;
    rp->adapt = adapt && !K.flat_proposal_dist;
    rp->rao_iz1 = rz1 > 0 ? 1.0 / rz1 : 0.0;
    rp->rao_z2 = rz2;
    rp->prop_iz1 = pz1 > 0 ? 1.0 / pz1 : 0.0;
    rp->prop_z2 = pz2;
    rp->inv_2s2 = 1.0 / (2 * M->sigma2);
    rp->scale = ldexp(1.0, -W.s.bulk_s);
    rp->mr = (double)W.s.bsuml[0] * ldexp(1.0, -W.s.bulk_s) / W.P.n;
    for (int t = 0; t < 4; ++t) {
      rp->itv[t] = ch->inv_t2a2[t];
      rp->nlog_itv[t] = -flog(ch->inv_t2a2[t]);
    }
    // the same constants as FP32 pairs for the double-float posterior
    rp->scale_f = (float)rp->scale;
    const dfl mr = df_from_double(rp->mr), i2s = df_from_double(rp->inv_2s2);
    rp->mr_df[0] = mr.h;
    rp->mr_df[1] = mr.l;
    rp->i2s_df[0] = i2s.h;
    rp->i2s_df[1] = i2s.l;
    for (int t = 0; t < 4; ++t) {
      const dfl v = df_from_double(rp->itv[t]);
      rp->itv_df[t][0] = v.h;
      rp->itv_df[t][1] = v.l;
    }
  }
  // log prior changes of the scan (src/sampler.cpp:51-76)
  int Ns[5];
  for (int t = 0; t < 5; ++t) Ns[t] = M->Ns[t];
  int nl = M->k;
  for (int t = 0; t < 5; ++t) {
    if (!K.allow_types[t]) continue;
    double la = 0;
    if ((uint64_t)(Ns[t] + 1) <= K.p) la = W.lchange_add(Ns, nl, t);
    if (W.lane == 0) {
      rp->lmp_add[t] = la;
      if (t < 4) {
        rp->cadd[t] = la - 0.5 * rp->nlog_itv[t];
        const dfl v = df_from_double(rp->cadd[t]);
        rp->cadd_df[t][0] = v.h;
        rp->cadd_df[t][1] = v.l;
      }
    }
    Ns[t]--;
    nl--;
    if (Ns[t] >= 0) {
      for (int j = 0; j < 5; ++j) {
        if (!K.allow_types[j]) continue;
        double lr = W.lchange_add(Ns, nl, j);
        if (W.lane == 0) rp->lmp_rem[t][j] = lr;
      }
    }
    Ns[t]++;
    nl++;
  }
  __syncwarp();
  if (!scan_only && adapt) {
    if (K.adapt_p_move_size) W.adapt_move_size();
    if (W.lane == 0) {
      ch->p_proposal_n++;
      if (!K.flat_proposal_dist) ch->rebuild = 1;
    }
  }
  // many pending flips make every proposal draw slower: ask the rebuild
  // that follows the scan for a fresh prefix
  if (!scan_only && W.lane == 0 && W.s.n_pend > BMG_PEND_REBUILD) ch->rebuild = 1;
  if (W.lane == 0) ch->rb_pending = do_scan || adapt;
  __syncwarp();
}

// ------------------------------------------------------------- kernels
// A move CTA's shared memory: ~190 KB, so it is dynamic (one CTA per SM).
struct MoveSmem {
  MoveShared s;
  BulkCols bc;
  long long part[BMG_MOVE_THREADS];
};
static_assert(sizeof(MoveSmem) <= 227 * 1024, "a move CTA's shared memory exceeds one SM's");

__device__ __forceinline__ MoveSmem& move_smem()
{
  extern __shared__ __align__(16) unsigned char bmg_move_dsm[];
  return *reinterpret_cast<MoveSmem*>(bmg_move_dsm);
}

template <class T>
__device__ void block_copy(T* dst, const T* src)
{
  static_assert(sizeof(T) % 4 == 0, "word copy");
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  const uint32_t* q = reinterpret_cast<const uint32_t*>(src);
  for (unsigned i = threadIdx.x; i < sizeof(T) / 4; i += blockDim.x) d[i] = q[i];
}

// All threads: chain c's dynamic state and both model headers into shared
// memory, with the factors and v of each model that fits in SMK.
__device__ void load_state(const DevConst& K, int c, MoveShared& s)
{
  block_copy(&s.chs, K.ch + c);
  block_copy(&s.mod[0], K.cur + c);
  block_copy(&s.mod[1], K.nm + c);
  block_copy(&s.phs, K.ph + K.pheno_of[c]);
  __syncthreads();
  for (int i = 0; i < 2; ++i) {
    const DevModel& M = s.mod[i];
    const bool on = M.llen <= SMK && M.vlen <= SMK && M.xcols <= SMK;
    if (on) {
      const size_t tri = (size_t)M.llen * (M.llen + 1) / 2;
      for (size_t q = threadIdx.x; q < tri; q += blockDim.x) s.Ls[i][q] = M.l[q];
      for (int q = threadIdx.x; q < M.vlen; q += blockDim.x) s.vs[i][q] = M.v[q];
    }
    if (threadIdx.x == 0) s.l_smem[i] = on;
  }
  __syncthreads();
}

// All threads: the inverse of load_state.
__device__ void store_state(const DevConst& K, int c, MoveShared& s)
{
  __syncthreads();
  for (int i = 0; i < 2; ++i) {
    const DevModel& M = s.mod[i];
    if (!s.l_smem[i]) continue;
    const int ll = min(M.llen, SMK);
    const size_t tri = (size_t)ll * (ll + 1) / 2;
    for (size_t q = threadIdx.x; q < tri; q += blockDim.x) M.l[q] = s.Ls[i][q];
    for (int q = threadIdx.x; q < min(M.vlen, SMK); q += blockDim.x) M.v[q] = s.vs[i][q];
  }
  block_copy(K.ch + c, &s.chs);
  block_copy(K.cur + c, &s.mod[0]);
  block_copy(K.nm + c, &s.mod[1]);
}

// Model of every chain at construction (src/model.hpp:49-113): the covariate
// block is set by the host; here its likelihood, then new = current.
extern "C" __global__ void __launch_bounds__(32)
bmg_init_kernel(DevConst K)
{
  MoveShared& s = move_smem().s;
  load_state(K, blockIdx.x, s);
  if (threadIdx.x == 0) s.err = 0;
  __syncwarp();
  Warp W(K, blockIdx.x, s);
  W.compute_log_likelihood(W.cur);
  W.copy_model(W.nm, W.cur);
  if (W.lane == 0 && s.err) W.ch->error = s.err;
  store_state(K, blockIdx.x, s);
}

// Residual limbs and RbParams of every chain at its current beta, for a scan
// requested outside the MCMC loop (bmg_scan).  With from_yhat the residual is
// y - K.yhat instead (K.yhat then holds the caller's fitted values for each
// chain, yhat_absmax their largest magnitude; bmg_scan_yhat).
extern "C" __global__ void __launch_bounds__(BMG_MOVE_THREADS, 1)
bmg_rbprep_kernel(DevConst K, int from_yhat, double yhat_absmax)
{
  MoveShared& s = move_smem().s;
  BulkCols& bc = move_smem().bc;
  const int c = blockIdx.x, tid = threadIdx.x;
  load_state(K, c, s);
  if (tid == 0) {
    s.err = 0;
    s.yhat_given_max = yhat_absmax;
  }
  __syncthreads();
  Warp W(K, c, s);
  if (tid < 32) bulk_setup(W, bc, BULK_RESID | (from_yhat ? BULK_YHAT : 0));
  __syncthreads();
  bulk_phase(K, c, s, bc);
  if (tid < 32) {
    prep_rb(W, true);
    if (W.lane == 0) s.chs.rng = W.rng;
  }
  store_state(K, c, s);
}

// The corrections of the RB scan for the SNPs with missing calls, one warp
// per (SNP, chain) that scans this step: outside the model the calls are
// imputed from their prior at the slots prep_rb reserved (src/sampler.cpp:
// 731-736, src/data_model.cpp:78-90; the values serve this scan only, a SNP
// that enters the model is imputed afresh), in the model their current
// values hold.  dxr = sum x_t(value) R_i over the calls, and the precomputed
// values as DataModel::update_prexx_cov corrects them (src/data_model.cpp:
// 105-167).  Grid (ceil(miss_snps / 8), chains) x 256 threads.
extern "C" __global__ void __launch_bounds__(256) bmg_miss_scan_kernel(DevConst K)
{
  const int c = blockIdx.y, lane = threadIdx.x & 31;
  const RbParams& rp = K.rb[c];
  if (!rp.do_scan) return;
  const uint32_t m = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (m >= K.miss_snps) return;
  const uint32_t j = K.miss_list[m];
  const long long o0 = K.miss_off[j], nmc = K.miss_off[j + 1] - o0;
  const bool inm = (K.inbits[(size_t)c * ((K.p + 31) / 32) + (j >> 5)] >> (j & 31)) & 1u;
  uint64_t base = 0;
  if (!inm) {
    // in-model SNPs below j and their missing calls
    const long long* il = K.miss_inm + (size_t)c * 2 * K.km;
    int lo = 0, hi = rp.n_inm;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if ((uint64_t)il[mid] < j) lo = mid + 1;
      else hi = mid;
    }
    base = rp.miss_slot + (uint64_t)(o0 - il[K.km + lo]);
  }
  const double* mp = K.miss_prior + 3 * (size_t)j;
  const int64_t* R = K.resid + (size_t)c * K.n_pad;
  long long dxr[4] = {0, 0, 0, 0};
  int sg[4] = {0, 0, 0, 0}, sg2[4] = {0, 0, 0, 0}, cr[4][4] = {{0}}, n1 = 0;
  for (long long q = lane; q < nmc; q += 32) {
    int v;
    if (inm) {
      v = K.miss_val[(size_t)c * K.miss_total + o0 + q];
    } else {
      v = miss_draw(mp, bmg_uniform01_at(rp.key0, rp.key1, base + (uint64_t)q));
    }
    const long long Ri = R[K.miss_ind[o0 + q]];
    n1 += (v == 1);
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int x = gval_term(v, t);
      dxr[t] += x * Ri;
      sg[t] += x;
      sg2[t] += x * x;
#pragma unroll
      for (int u = 0; u < 4; ++u) cr[t][u] += x * gval_term(v, u);
    }
  }
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    dxr[t] = warp_sum_ll(dxr[t]);
    sg[t] = warp_sum_i(sg[t]);
    sg2[t] = warp_sum_i(sg2[t]);
#pragma unroll
    for (int u = 0; u < 4; ++u) cr[t][u] = warp_sum_i(cr[t][u]);
  }
  n1 = warp_sum_i(n1);
  if (lane != 0) return;
  MissCorr& mc = K.miss_corr[(size_t)c * K.miss_snps + m];
  const DevPheno& P = K.ph[K.pheno_of[c]];
  const double* pre = P.pre + (size_t)j * K.offset;
  double pc[BMG_MAX_OFFSET];
  for (int q = 0; q < K.offset; ++q) pc[q] = pre[q];
  const double nn = P.n;
  double* loc = pc;
  const bool ah = K.allow_types[4];
  const double sah = ah ? pc[0] * pc[2] : 0.0;
  for (int t = 0; t < 4; ++t) {
    if (!K.allow_terms[t]) continue;
    const double old_sum = loc[0];
    loc[0] += sg[t];
    loc[1] += sg2[t] - sg[t] * (old_sum * 2.0 + sg[t]) / nn;
    loc += 2;
  }
  if (ah) {
    loc[0] += (sah - pc[0] * pc[2]) / nn;
    loc[0] += (double)n1;
  }
  for (int q = 0; q < K.offset; ++q) mc.pre[q] = pc[q];
  for (int t = 0; t < 4; ++t) {
    mc.dxr[t] = dxr[t];
    mc.dsum[t] = sg[t];
    for (int u = 0; u < 4; ++u) mc.dcross[t][u] = cr[t][u];
  }
}

// Every chain's current sigma2 (bmg_scan_yhat)
extern "C" __global__ void bmg_set_sigma2_kernel(DevConst K, double sigma2)
{
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < K.n_chains) K.cur[c].sigma2 = sigma2;
}

// Runs iterations of chain blockIdx.x until `max_iters` are done or an RB
// step has been prepared (its residual limbs and RbParams written).
extern "C" __global__ void __launch_bounds__(BMG_MOVE_THREADS, 1)
bmg_move_kernel(DevConst K, int max_iters)
{
  MoveShared& s = move_smem().s;
  BulkCols& bc = move_smem().bc;
  long long* part = move_smem().part;
  const int c = blockIdx.x;
  const int tid = threadIdx.x;
  load_state(K, c, s);
  DevChain* ch = &s.chs;
  if (tid == 0) {
    s.err = ch->error;
    s.n_pend = ch->n_pend;
    s.iter_stop = 0;
  }
  __syncthreads();
  if (s.err) return;
  for (int i = tid; i < s.n_pend; i += blockDim.x) {
    int sn = ch->pend_snp[i];
    s.pend_snp[i] = sn;
    s.pend_pos[i] = K.pos[sn];
    double pp = K.p_prop[(size_t)c * K.p + K.pos[sn]];
    long long w = __double2ll_rn(fmax(pp, K.q_add_min) * ldexp(1.0, K.qs));
    bool bz = (K.basebits[(size_t)c * ((K.p + 31) / 32) + (sn >> 5)] >> (sn & 31)) & 1u;
    s.pend_d[i] = bz ? w : -w;
  }
  __syncthreads();

  // warp 0 keeps the sampler context (and its random stream) in registers
  Warp W(K, c, s);
  if (K.lrn.on && tid < 32) W.mlp_init_total();
  double* cs_buf = K.scratch + (size_t)c * 2 * K.km;
  double* sn_buf = cs_buf + K.km;

  if (tid < 32 && !ch->started) {
    /* src/sampler.cpp:551-620: the model is still empty here, so alpha is
       drawn from its prior and needs no data pass */
    if (!isfinite(W.cur->ll)) W.fail(BMG_DERR_START);
    W.copy_model(W.nm, W.cur);
    W.sample_beta_sigma2(W.cur);
    W.sample_tau2(W.cur);
    double a = W.sample_alpha(W.cur, 0.0, 0.0);
    W.set_alpha(a, W.cur);
    W.compute_log_likelihood(W.cur);
    W.copy_model(W.nm, W.cur);
    if (W.lane == 0) ch->started = 1;
  }
  __syncthreads();

  for (int it = 0; it < max_iters; ++it) {
    __syncthreads();
    if (s.err || s.iter_stop) break;
    // room for one more move's flips of dd_add, else rebuild its prefix here
    if (s.n_pend > BMG_PEND_MAX - 2 * (int)K.max_move_size - 2) {
      if (tid == 0) ch->n_pend = 0;
      rebuild_chain(K, c, part, ch);
      if (tid == 0) s.n_pend = 0;
      __syncthreads();
    }
    const uint64_t iter = ch->n_iter;
    const bool ns_step = ((iter + 1) % K.n_sample_tau2) == 0;
    const bool thin_step = ((iter + 1) % K.thin) == 0;
    const bool rb_step = ((iter + 1) % K.n_rao) == 0;
    if (ns_step) {
      /* src/sampler.cpp:628-635 */
      if (tid < 32) {
        W.sample_missing_gibbs();
        bulk_setup(W, bc, BULK_ALPHA);
      }
      __syncthreads();
      bulk_phase(K, c, s, bc);
      if (tid < 32) {
        W.sample_tau2(W.cur);
        double a = W.sample_alpha(W.cur, s.bsum[1], s.bsum[2]);
        W.set_alpha(a, W.cur);
        W.compute_log_likelihood(W.cur);
        W.copy_model(W.nm, W.cur);
      }
      __syncthreads();
    }
    if (tid < 32) {
      /* src/sampler.cpp:637-684; move mix of compute_p_moves (:455-515) */
      double pm[7], pcs[7];
      if (K.n_types > 1) { pm[0] = 0.8; pm[1] = 0.1; pm[2] = 0.0; pm[3] = 0.1; }
      else { pm[0] = 0.7; pm[1] = 0.15; pm[2] = 0.15; pm[3] = 0.0; }
      pm[4] = pm[5] = pm[6] = 0.0;
      pcs[0] = pm[0];
      for (int i = 1; i < 7; ++i) pcs[i] = pcs[i - 1] + pm[i];
      int move = W.sample_naive(pcs, 7);
      int jd = 0;
      W.helpers = true;
      switch (move) {
        case 0: jd = W.do_addrem_move(cs_buf, sn_buf); break;
        case 1:
          if (W.cur->k > 0 && (long long)W.cur->k < (long long)K.p - 1) jd = W.do_swap_move(cs_buf, sn_buf);
          break;
        case 2:
          if (W.cur->k > 0 && K.p > 2) jd = W.do_statechange_move(cs_buf, sn_buf);
          break;
        case 3:
          if (W.cur->k > 0) jd = W.do_typeswitch_move(cs_buf, sn_buf);
          break;
        default: W.fail(BMG_DERR_NAN); break;
      }
      W.help_exit();
      if (W.lane == 0) {
        ch->n_moves[move]++;
        ch->n_acpt[move] += (jd > 0);
        ch->n_accepted += (jd > 0);
      }
      __syncwarp();
      const bool pre_ns = ((iter + 2) % K.n_sample_tau2) == 0;
      if (thin_step || pre_ns) W.sample_beta_sigma2(W.cur);
      if (W.lane == 0) {
        uint32_t ti = ch->tr_iter;
        if (ti < K.tr.iter_cap) {
          size_t o = (size_t)c * K.tr.iter_cap + ti;
          K.tr.jump[o] = (uint8_t)jd;
          K.tr.mtype[o] = (uint8_t)move;
          K.tr.msize[o] = (uint8_t)ch->movesize;
          ch->tr_iter = ti + 1;
        } else if (s.err == 0) {
          s.err = BMG_DERR_TRACE;
        }
      }
      __syncwarp();
      if (thin_step) bulk_setup(W, bc, BULK_PVE | (rb_step ? BULK_RESID : 0));
    } else {
      help_loop(K, s);
    }
    __syncthreads();
    if (thin_step) {
      bulk_phase(K, c, s, bc);
      if (tid < 32) {
        /* src/sampler.cpp:691-727, src/model.hpp:345-392 */
        DevModel* M = W.cur;
        const double n = s.phs.n;
        const bool ce = K.m_e > 1, cg = M->k > 0;
        double pv[3];
        double vg = (s.bsum[1] - s.bsum[0] * s.bsum[0] / n) / (n - 1);
        double ve = (s.bsum[3] - s.bsum[2] * s.bsum[2] / n) / (n - 1);
        double vt = (s.bsum[5] - s.bsum[4] * s.bsum[4] / n) / (n - 1);
        pv[2] = ce ? ve : 0.0;
        pv[1] = cg ? vg : 0.0;
        if (ce || cg) {
          pv[0] = !ce ? pv[1] : (!cg ? pv[2] : vt);
          double z = pv[0] + M->sigma2;
          pv[0] /= z; pv[1] /= z; pv[2] /= z;
        } else {
          pv[0] = pv[1] = pv[2] = 0;
        }
        double lp = W.log_model(M->Ns);
        uint32_t tt = ch->tr_thin, tl = ch->tr_loci;
        bool room = tt < K.tr.thin_cap && tl + M->k <= K.tr.loci_cap;
        if (W.lane == 0) {
          ch->pves[0] = pv[0]; ch->pves[1] = pv[1]; ch->pves[2] = pv[2];
          if (room) {
            size_t o = (size_t)c * K.tr.thin_cap + tt;
            K.tr.msz[o] = M->k;
            K.tr.ll[o] = M->ll;
            K.tr.lp[o] = lp;
            K.tr.s2[o] = M->sigma2;
            K.tr.alpha[o] = ch->alpha;
            K.tr.pve[3 * o] = pv[0];
            K.tr.pve[3 * o + 1] = pv[1];
            K.tr.pve[3 * o + 2] = pv[2];
            ch->tr_thin = tt + 1;
            ch->tr_loci = tl + M->k;
          } else if (s.err == 0) {
            s.err = BMG_DERR_TRACE;
          }
        }
        if (room) {
          for (int i = W.lane; i < M->k; i += 32) {
            K.tr.loci[(size_t)c * K.tr.loci_cap + tl + i] = M->loci[i];
            K.tr.types[(size_t)c * K.tr.loci_cap + tl + i] = M->type_inds[i];
          }
        }
        if (K.save_beta) {
          uint32_t tb = ch->tr_beta;
          if (tb + M->blen <= K.tr.beta_cap) {
            for (int i = W.lane; i < M->blen; i += 32) K.tr.beta[(size_t)c * K.tr.beta_cap + tb + i] = M->beta[i];
            __syncwarp();
            if (W.lane == 0) ch->tr_beta = tb + M->blen;
          } else if (W.lane == 0 && s.err == 0) {
            s.err = BMG_DERR_TRACE;
          }
        }
        __syncwarp();
      }
    }
    __syncthreads();
    if (tid < 32) {
      if (rb_step) {
        prep_rb(W, false);
        if (W.lane == 0) s.iter_stop = 1;
      }
      if (K.verbosity > 0 && ((iter + 1) % K.verbosity) == 0) {
        /* src/sampler.cpp:813-833 */
        double lp = W.log_model(W.cur->Ns);
        if (W.lane == 0) {
          uint32_t tg = ch->tr_log;
          if (tg < K.tr.log_cap) {
            double* r = K.tr.logrec + ((size_t)c * K.tr.log_cap + tg) * BMG_LOGREC;
            r[0] = (double)(iter + 1);
            r[1] = (double)ch->n_accepted;
            r[2] = (double)ch->n_acpt[1];
            r[3] = (double)ch->n_moves[1];
            r[4] = (double)ch->n_acpt[2];
            r[5] = (double)ch->n_moves[2];
            r[6] = ch->p_move_size;
            r[7] = (double)W.cur->k;
            r[8] = W.cur->ll + lp;
            r[9] = ch->pves[0];
            r[10] = ch->pves[1];
            r[11] = ch->pves[2];
            r[12] = W.cur->sigma2;
            ch->tr_log = tg + 1;
          }
        }
      }
      if (W.lane == 0) {
        ch->n_iter = iter + 1;
        if (s.err) ch->error = s.err;
      }
      __syncwarp();
    }
  }
  __syncthreads();
  if (tid == 0) {
    ch->rng = W.rng;
    ch->n_pend = s.n_pend;
    for (int i = 0; i < s.n_pend; ++i) ch->pend_snp[i] = s.pend_snp[i];
    if (s.err) ch->error = s.err;
  }
  store_state(K, c, s);
}

// dynamic shared memory of the three kernels above
extern "C" cudaError_t bmg_move_configure(size_t* smem_bytes)
{
  const int bytes = (int)sizeof(MoveSmem);
  cudaError_t e = cudaFuncSetAttribute(bmg_init_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(bmg_rbprep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(bmg_move_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (smem_bytes) *smem_bytes = sizeof(MoveSmem);
  return e;
}
