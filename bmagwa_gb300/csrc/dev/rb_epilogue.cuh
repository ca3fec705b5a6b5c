// The Rao-Blackwell epilogue shared by both scan implementations: from the
// exact products x_t(j)' r of one (SNP, chain) to the reference's single-SNP
// posterior (src/sampler.cpp:89-258) and the running means (:739-776).
#ifndef BMG_RB_EPILOGUE_CUH_
#define BMG_RB_EPILOGUE_CUH_

#include <math.h>

#include "common.cuh"
#include "exp_table.h"
#include "rb_df.h"

static __device__ __forceinline__ bool in_model(const DevConst& K, int c, uint64_t j)
{
  return (K.inbits[(size_t)c * ((K.p + 31) / 32) + (j >> 5)] >> (j & 31)) & 1u;
}

// a SNP outside the model and without missing calls: the fast posterior
// applies (SNPs with missing calls take rb_epilogue and their corrections)
static __device__ __forceinline__ bool rb_plain(const DevConst& K, int c, uint64_t j)
{
  return !in_model(K, c, j) && !(K.miss_total && K.miss_rank[j] >= 0);
}

// The common case: one non-AH effect type and the chain's shared tau2.  For
// a SNP outside the model the posterior needs no branch, so a thread can
// evaluate two (SNP, chain) units back to back and their FP64 chains overlap.
// The expressions are those of rb_epilogue below, term by term.
static __device__ __forceinline__ bool rb_fast_ok(const DevConst& K)
{
  return !K.use_individual_tau2 && K.n_types == 1 && K.types[0] != 4;
}

// exp(a) for |a| <= 700 by Tang's table-driven method (P. T. P. Tang,
// "Table-driven implementation of the exponential function in IEEE
// floating-point arithmetic", ACM TOMS 15(2), 1989).  a = k ln2/256 + r with
// k = 256 m + i and |r| <= ln2/512, so exp(a) = 2^m 2^(i/256) exp(r).  The
// reduction splits ln2/256 into a 34-bit head (k head exact for |k| < 2^19)
// and a tail; exp(r) is its Taylor series to r^4 (truncation below 4e-17
// relative).  Nine FP64 instructions; the 2^m scaling is an integer add to the
// exponent field, valid because the result stays a normal number.
static __device__ __forceinline__ double bmg_exp_tab(double a)
{
  const double shift = 0x1.8p52;  // adding it rounds a 256/ln2 to an integer in the low word
  const double ks = fma(a, 0x1.71547652b82fep+8, shift);
  const int k = __double2loint(ks);
  const double kd = ks - shift;
  double r = fma(-kd, 0x1.62e42fef80000p-9, a);
  r = fma(-kd, 0x1.1cf79abc9e3b4p-44, r);
  const double q = fma(fma(fma(1.0 / 24, r, 1.0 / 6), r, 0.5), r, 1.0);  // (exp(r) - 1) / r
  const double t = __ldg(&kExp2Tab[k & 255]);
  const double y = fma(t, r * q, t);
  return __hiloint2double(__double2hiint(y) + ((k >> 8) << 20), __double2loint(y));
}

// p_r of (SNP j, chain c) from the exact product xi = x_t(j)' R_c; *lo gets
// the log posterior odds of inclusion when the scan keeps them (K.p_lml).
static __device__ __forceinline__ double rb_fast_pr(const DevConst& K, int c, uint64_t j, long long xi, double* lo)
{
  const RbParams& rp = K.rb[c];
  const DevPheno& P = K.ph[K.pheno_of[c]];
  const int type = K.types[0];
  if (!K.p_lml && P.pre_f && rp.scale_f >= 0x1p-100f) {
    // double-float arithmetic (relative error below 1e-12); FP64 below
    const float4 pf = __ldg(&P.pre_f[j]);
    const double pr = rb_pr_df(xi, rp.scale_f, pf.x, dfl{pf.y, pf.z}, dfl{rp.mr_df[0], rp.mr_df[1]},
                               dfl{rp.itv_df[type][0], rp.itv_df[type][1]}, dfl{rp.i2s_df[0], rp.i2s_df[1]},
                               dfl{rp.cadd_df[type][0], rp.cadd_df[type][1]}, kExp2TabF);
    if (pr >= 0) {
      *lo = 0;
      return pr;
    }
  }
  const double* pre = P.pre + j * (size_t)K.offset;
  const int off = K.offset_type[type];
  const double xr = (double)xi * rp.scale;
  const double det = pre[off + 1] + rp.itv[type];
  const double rx = xr - pre[off] * rp.mr;
  if (K.p_lml) {
    // the reference's expression term by term, log odds kept
    const double slq = rp.nlog_itv[type];
    const double et = (rx * rx) / det;
    const double p = et * rp.inv_2s2 - 0.5 * (log(det) + slq) + rp.lmp_add[type];
    *lo = p;
    const double e = exp(p);
    return isfinite(e) ? e / (1 + e) : 1;
  }
  // the same odds without the log: with s = det^-1/2, rx^2/det = (rx s)^2 and
  // exp(p) = exp(et/(2 sigma2) + lmp - slq/2) s.  Odds above 2^54 round
  // p_r to 1 (a > 700 included, with NaN as the reference maps it); a < -700
  // takes the library exp.
  *lo = 0;
  const double s = rsqrt(det);
  const double t = rx * s;
  const double a = fma(t * t, rp.inv_2s2, rp.cadd[type]);
  if (!(a <= 700.0)) return 1;
  double ea;
  if (a >= -700.0)
    ea = bmg_exp_tab(a);
  else
    ea = exp(a);
  const double e = ea * s;
  return e / (1 + e);
}

// p_r and the running means of one (SNP, chain) with one effect type
// (src/sampler.cpp:739-776)
static __device__ __forceinline__ void rb_store1(const DevConst& K, int c, uint64_t j, double pr, double lo)
{
  const RbParams& rp = K.rb[c];
  const size_t cj = (size_t)c * K.p + j;
  if (K.p_r) K.p_r[cj] = pr;
  if (K.p_lml) K.p_lml[cj] = lo;
  if (rp.acc_rao) K.p_rao[cj] = fma(rp.rao_z2, K.p_rao[cj], pr * rp.rao_iz1);
  if (rp.adapt) {
    const size_t q = (size_t)c * K.p + K.pos[j];
    K.p_prop[q] = fma(rp.prop_z2, K.p_prop[q], pr * rp.prop_iz1);
  }
}

// xr[t] = x_t(j)' R_c for term type t (A,H,D,R), exact, residual scale 2^-s.
// Writes p_r and updates the running means (src/sampler.cpp:739-776).
static __device__ __noinline__ void rb_epilogue(const DevConst& K, int c, uint64_t j, const long long* xr_by_type)
{
  const RbParams& rp = K.rb[c];
  const DevPheno& P = K.ph[K.pheno_of[c]];
  const double n = P.n;
  // the SNP's missing calls at their imputed values (DataModel overlay,
  // src/data_model.cpp:30-72, and update_prexx_cov, :105-167)
  const MissCorr* mc = nullptr;
  if (K.miss_total && K.miss_rank[j] >= 0) mc = &K.miss_corr[(size_t)c * K.miss_snps + K.miss_rank[j]];
  double xr[4];
  for (int t = 0; t < 4; ++t)
    xr[t] = K.allow_terms[t] ? (double)(xr_by_type[t] + (mc ? mc->dxr[t] : 0ll)) * rp.scale : 0.0;
  double mr = rp.mr;
  double itv[4] = {rp.itv[0], rp.itv[1], rp.itv[2], rp.itv[3]};
  if (K.use_individual_tau2) {
    // Prior::sample_single_inv_tau2_from_prior_times_alpha2 (src/prior.hpp:192-199)
    // with Rand::rand_sinvchi2(nu, s2) (src/rand.hpp:85-97); slot of (j, term u)
    uint64_t slot = rp.rng_slot + j * (uint64_t)K.n_terms;
    for (int t = 0; t < 4; ++t) {
      if (!K.allow_terms[t]) continue;
      double nu = K.nu_tau2[t];
      double g = bmg_gamma_at(rp.key0, rp.key1, slot++, 0.5 * nu);
      double val = nu * K.s2_tau2[t] / (2.0 * g);
      itv[t] = 1.0 / (rp.alpha2 * val);
    }
  }
  const double* lmp = rp.lmp_add;
  // -log(itv[t]) of the shared tau2 is the chain's constant; per-SNP draws
  // and in-model precisions need their own
  bool own_itv = K.use_individual_tau2;
  if (in_model(K, c, j)) {
    const DevModel& M = K.cur[c];
    int mi = K.model_inds[(size_t)c * K.p + j];
    int type = K.types[M.type_inds[mi]];
    int x1 = M.x_ind1[mi];
    int t1 = M.xc_type[x1];
    double b1 = M.beta[x1];
    if (K.use_individual_tau2) {
      if (type == 4) { itv[0] = M.inv[x1]; itv[1] = M.inv[M.x_ind2[mi]]; }
      else itv[type] = M.inv[x1];
    }
    // r_om = r + x_j beta_j: products and mean from the genotype counts
    // (and the imputed values of the missing calls)
    double msum = b1 * (double)(term_sum(P.cnt, j, t1) + (mc ? mc->dsum[t1] : 0));
    for (int t = 0; t < 4; ++t)
      if (K.allow_terms[t]) xr[t] += b1 * (double)(term_cross_same(P.cnt, j, t, t1) + (mc ? mc->dcross[t][t1] : 0));
    if (type == 4) {
      int x2 = M.x_ind2[mi];
      int t2 = M.xc_type[x2];
      double b2 = M.beta[x2];
      msum += b2 * (double)(term_sum(P.cnt, j, t2) + (mc ? mc->dsum[t2] : 0));
      for (int t = 0; t < 4; ++t)
        if (K.allow_terms[t]) xr[t] += b2 * (double)(term_cross_same(P.cnt, j, t, t2) + (mc ? mc->dcross[t][t2] : 0));
    }
    mr = mr + msum / n;
    lmp = rp.lmp_rem[type];
  }
  const double* pre = mc ? mc->pre : P.pre + j * (size_t)K.offset;
  const int nt = K.n_types;
  const bool ut = nt > 1;
  double pt[5];
  double pr = 0, lo = 0;
  double maxt = -INFINITY;
  for (int t = 0; t < nt; ++t) {
    int type = K.types[t];
    double det, et, slq;
    if (type == 4) {
      double sa = pre[0], va = pre[1] + itv[0], sh = pre[2], vh = pre[3] + itv[1];
      double vah = pre[K.offset - 1];
      slq = own_itv ? -log(itv[0]) - log(itv[1]) : rp.nlog_itv[0] - log(itv[1]);
      double rxa = xr[0] - sa * mr;
      double rxh = xr[1] - sh * mr;
      det = va * vh - vah * vah;
      et = rxa * rxa * vh - 2.0 * rxa * rxh * vah + rxh * rxh * va;
      et /= det;
    } else {
      int off = K.offset_type[type];
      double sv = pre[off];
      det = pre[off + 1] + itv[type];
      slq = own_itv ? -log(itv[type]) : rp.nlog_itv[type];
      double rx = xr[type] - sv * mr;
      et = (rx * rx) / det;
    }
    double p = et * rp.inv_2s2 - 0.5 * (log(det) + slq) + lmp[type];
    if (ut) {
      if (p > maxt) maxt = p;
      pt[t] = p;
    } else {
      lo = p;
      double e = exp(p);
      pr = isfinite(e) ? e / (1 + e) : 1;
    }
  }
  if (ut) {
    if (!isfinite(maxt)) {
      if (maxt > 0) {
        double st = 0;
        for (int t = 0; t < nt; ++t) { pt[t] = (!isfinite(pt[t]) && pt[t] > 0) ? 1 : 0; st += pt[t]; }
        for (int t = 0; t < nt; ++t) pt[t] /= st;
        pr = 1;
      } else {
        for (int t = 0; t < nt; ++t) pt[t] = 1.0 / nt;
        pr = 0;
      }
      if (isnan(maxt)) atomicExch(&K.ch[c].error, BMG_DERR_NAN);
      lo = maxt;
    } else {
      double st = 0;
      for (int t = 0; t < nt; ++t) { pt[t] = exp(pt[t] - maxt); st += pt[t]; }
      for (int t = 0; t < nt; ++t) pt[t] /= st;
      lo = log(st) + maxt;
      st = exp(log(st) + maxt);
      pr = isfinite(st) ? st / (1 + st) : 1;
    }
  }
  const size_t cj = (size_t)c * K.p + j;
  if (K.p_lml) K.p_lml[cj] = lo;
  if (K.p_r) {
    K.p_r[cj] = pr;
    if (ut)
      for (int t = 0; t < nt; ++t) K.p_r_types[cj * nt + t] = pt[t];
  }
  if (rp.acc_rao) {
    K.p_rao[cj] = fma(rp.rao_z2, K.p_rao[cj], pr * rp.rao_iz1);
    if (ut)
      for (int t = 0; t < nt; ++t)
        K.p_rao_types[cj * nt + t] = fma(rp.rao_z2, K.p_rao_types[cj * nt + t], pt[t] * rp.rao_iz1);
  }
  if (rp.adapt) {
    size_t q = (size_t)c * K.p + K.pos[j];
    K.p_prop[q] = fma(rp.prop_z2, K.p_prop[q], pr * rp.prop_iz1);
    if (ut)
      for (int t = 0; t < nt; ++t)
        K.p_prop_types[cj * nt + t] = fma(rp.prop_z2, K.p_prop_types[cj * nt + t], pt[t] * rp.prop_iz1);
  }
}

#endif
