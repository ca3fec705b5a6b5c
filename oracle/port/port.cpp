/*
 * oracle/port/port.cpp -- CPU restatement of bmagwa's MCMC over SNP inclusion.
 *
 * ORACLE / TEST INFRASTRUCTURE (see port.h).  Every function names the
 * reference lines it restates.  The floating-point order follows the
 * reference (sequential dots of oracle/linalg.c, same update formulas), and
 * random numbers come from include/bmg_rng.h in the reference's draw order.
 */
#include "port.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "bmg_rng.h"
#include "../shim/cblas.h"

extern "C" void dpotrf_(char* uplo, int* n, double* a, int* lda, int* info);
extern "C" void dchex_(double* r, int* ldr, int* p, int* k, int* l, double* z,
                       int* ldz, int* nz, double* c, double* s, int* job);

namespace bmgport_impl {

enum ef_t { A = 0, H = 1, D = 2, R = 3, AH = 4 };
static const double kLogHalf = -0.69314718055994528622676398299518041312694549560546875;

static double ddot(size_t n, const double* x, const double* y)
{
  return cblas_ddot((int)n, x, 1, y, 1);
}

/* ---------------------------------------------------------------- random */
/* src/rand.hpp:36-191 on the stream of bmg_rng.h */
struct Rand {
  bmg_rng_t st;
  double sinvchi2_nu, gamma_alpha;
  Rand(uint32_t seed, double nu) : sinvchi2_nu(nu), gamma_alpha(0.5 * nu)
  {
    bmg_rng_init(&st, seed);
  }
  double rand_01() { return bmg_uniform01(&st); }
  double rand_normal() { return bmg_normal(&st); }
  /* src/rand.hpp:61-78 */
  double rand_sinvchi2(double s2)
  {
    double val = -1.0;
    while (val <= 0 || !std::isfinite(val)) {
      val = sinvchi2_nu * s2 / (2.0 * bmg_gamma(&st, gamma_alpha));
    }
    return val;
  }
  /* src/rand.hpp:85-97 */
  double rand_sinvchi2(double nu, double s2)
  {
    double val = -1.0;
    while (val <= 0 || !std::isfinite(val)) {
      val = nu * s2 / (2.0 * bmg_gamma(&st, 0.5 * nu));
    }
    return val;
  }
};

/* src/utils.cpp:46-57 */
static int sample_discrete_naive(const double* cumsum, int m, Rand& rng)
{
  double z = cumsum[m - 1];
  double r = rng.rand_01() * z;
  for (int i = 0; i < m; ++i)
    if (r < cumsum[i]) return i;
  throw std::logic_error("sample_discrete_naive reached end");
}

/* src/utils.cpp:73-101: `level` bisection steps, then a linear search */
static size_t sample_discrete(const double* cumsum, size_t m, int level, Rand& rng)
{
  size_t a = 0, b = m - 1, c;
  double z = cumsum[b];
  double r = rng.rand_01() * z;
  while (level > 0) {
    c = (a + b) / 2;
    if (r < cumsum[c]) b = c;
    else a = c + 1;
    --level;
  }
  for (size_t i = a; i <= b; ++i)
    if (r < cumsum[i]) return i;
  throw std::logic_error("sample_discrete reached end");
}

/* src/utils.cpp:144-152 */
static void geometric_dist_cdf(int maxsize, double p, double* values)
{
  double q = 1 - p, qp = q;
  for (int i = 0; i < maxsize; ++i) {
    values[i] = 1 - q;
    q *= qp;
  }
}

/* ------------------------------------------------------------------ data */
struct Data {
  size_t n, m_g, m_e;  /* m_e counts the constant column (src/data.hpp:49) */
  size_t stride, n4;
  std::vector<double> y, e;  /* e: n x m_e, column 0 = 1 */
  std::vector<uint8_t> g;
  std::vector<std::vector<size_t> > miss_loc;   /* empty = no missing */
  std::vector<std::vector<double> > miss_prior; /* cumulative counts, 3 */
  double var_x, mean_x, var_y, yy;

  /* 2-bit code -> value, src/data.cpp:36-54 and src/genotype_tables.hpp */
  static double code_value(int code, int type)
  {
    if (code == 1) return -1.0;                 /* missing in every table */
    int gval = (code == 0) ? 0 : (code == 2 ? 1 : 2);
    switch (type) {
      case A: return (double)gval;
      case H: return (double)(gval == 1);
      case D: return (double)(gval > 0);
      default: return (double)(gval == 2);
    }
  }
  double get_genotype(size_t ind, size_t snp) const
  {
    uint8_t b = g[stride * snp + ind / 4];
    return code_value((b >> (2 * (ind % 4))) & 3, A);
  }
  void set_genotype(size_t ind, size_t snp, double v)
  {
    int code = (v == -1.0) ? 1 : (v == 0.0) ? 0 : (v == 1.0) ? 2 : 3;
    uint8_t& b = g[stride * snp + ind / 4];
    int sh = 2 * (int)(ind % 4);
    b = (uint8_t)((b & ~(3 << sh)) | (code << sh));
  }
  /* src/data.cpp:56-138 */
  /* four individuals per code byte from a table per term (the reference's
     genotype_tables.hpp lookups); the values are code_value()'s */
  void get_genotypes(int type, size_t snp, double* v) const
  {
    static double tab[4][256][4];
    static bool ready = false;
    if (!ready) {
      for (int t = 0; t < 4; ++t)
        for (int b = 0; b < 256; ++b)
          for (int q = 0; q < 4; ++q) tab[t][b][q] = code_value((b >> (2 * q)) & 3, t);
      ready = true;
    }
    const uint8_t* row = &g[stride * snp];
    const size_t full = n / 4;
    for (size_t w = 0; w < full; ++w) {
      const double* e = tab[type][row[w]];
      v[4 * w] = e[0];
      v[4 * w + 1] = e[1];
      v[4 * w + 2] = e[2];
      v[4 * w + 3] = e[3];
    }
    for (size_t i = 4 * full; i < n; ++i) v[i] = code_value((row[i / 4] >> (2 * (i % 4))) & 3, type);
  }

  Data(size_t n_, size_t m_g_, size_t m_e_, const uint8_t* packed, const double* y_,
       const double* e_, bool recode)
  : n(n_), m_g(m_g_), m_e(m_e_ + 1), stride((n_ + 3) / 4), n4(n_ / 4)
  {
    y.assign(y_, y_ + n);
    e.assign(n * m_e, 1.0);
    for (size_t j = 1; j < m_e; ++j)
      for (size_t i = 0; i < n; ++i) e[j * n + i] = e_[(j - 1) * n + i];
    g.assign(packed, packed + stride * m_g);
    if (recode) recode_g_to_minor_allele_count();
    handle_missing_g();
    yy = ddot(n, y.data(), y.data());
    /* Vector::var, src/vector.cpp:113-124 */
    double sq = 0, s = 0;
    for (size_t i = 0; i < n; ++i) { sq += y[i] * y[i]; s += y[i]; }
    var_y = (sq - s * s / n) / (n - 1);
    compute_g_var_and_mean();
  }
  /* src/data.cpp:324-339, src/utils.cpp:33-44 */
  void recode_g_to_minor_allele_count()
  {
    std::vector<double> col(n);
    for (size_t snp = 0; snp < m_g; ++snp) {
      get_genotypes(A, snp, col.data());
      double macount = 0;
      size_t ngenos = 0;
      for (size_t i = 0; i < n; ++i)
        if (col[i] >= 0) { macount += col[i]; ++ngenos; }
      if (macount / (2.0 * ngenos) > 0.5) {
        for (size_t ind = 0; ind < n; ++ind) {
          double gv = get_genotype(ind, snp);
          if (gv == 0.0) set_genotype(ind, snp, 2.0);
          else if (gv == 2.0) set_genotype(ind, snp, 0.0);
        }
      }
    }
  }
  /* src/data.cpp:341-376 */
  void handle_missing_g()
  {
    miss_loc.assign(m_g, std::vector<size_t>());
    miss_prior.assign(m_g, std::vector<double>());
    for (size_t snp = 0; snp < m_g; ++snp) {
      size_t nm = 0;
      for (size_t ind = 0; ind < n; ++ind)
        if (get_genotype(ind, snp) < 0) ++nm;
      if (nm == 0) continue;
      miss_prior[snp].assign(3, 0.0);
      for (size_t ind = 0; ind < n; ++ind) {
        double gv = get_genotype(ind, snp);
        if (gv < 0) miss_loc[snp].push_back(ind);
        else ++miss_prior[snp][(int)gv];
      }
      miss_prior[snp][1] += miss_prior[snp][0];
      miss_prior[snp][2] += miss_prior[snp][1];
    }
  }
  /* src/data.cpp:403-434 */
  void compute_g_var_and_mean()
  {
    double total_var = 0, total_mean = 0;
    size_t nm = 0, nv = 0;
    for (size_t snp = 0; snp < m_g; ++snp) {
      double sq = 0, s = 0;
      size_t ng = 0;
      for (size_t ind = 0; ind < n; ++ind) {
        double gv = get_genotype(ind, snp);
        if (gv >= 0) { sq += gv * gv; s += gv; ++ng; }
      }
      if (ng > 1) {
        total_mean += s / ng;
        total_var += (sq - s * s / ng) / (ng - 1);
        ++nm; ++nv;
      } else if (ng == 1) {
        total_mean += s / ng;
        ++nm;
      }
    }
    var_x = total_var / nv;
    mean_x = total_mean / nm;
  }
};

/* ------------------------------------------------------------- data model */
/* src/data_model.hpp:37-154, src/data_model.cpp:28-167 */
struct DataModel {
  const Data* data;
  size_t n, m_g, m_e, n_types;
  std::vector<int> types;
  bool allow_types_[5], allow_terms_[5];
  std::vector<std::vector<char> > miss_val;  /* per chain copy */

  DataModel(const Data* d, const std::vector<int>& t)
  : data(d), n(d->n), m_g(d->m_g), m_e(d->m_e), n_types(t.size()), types(t)
  {
    for (int i = 0; i < 5; ++i) allow_types_[i] = allow_terms_[i] = false;
    for (size_t i = 0; i < n_types; ++i) {
      allow_types_[types[i]] = true;
      if (types[i] == AH) { allow_terms_[A] = true; allow_terms_[H] = true; }
      else allow_terms_[types[i]] = true;
    }
    miss_val.resize(m_g);
    for (size_t i = 0; i < m_g; ++i)
      if (!d->miss_loc[i].empty()) miss_val[i].assign(d->miss_loc[i].size(), 0);
  }
  bool allow_types(int t) const { return allow_types_[t]; }
  bool allow_terms(int t) const { return allow_terms_[t]; }
  bool genotype_missing(size_t ind, size_t snp) const { return data->get_genotype(ind, snp) < 0; }
  /* src/data_model.cpp:30-72 */
  void get_genotypes(int type, size_t snp, double* v) const
  {
    data->get_genotypes(type, snp, v);
    const std::vector<size_t>& ml = data->miss_loc[snp];
    for (size_t i = 0; i < ml.size(); ++i) {
      int val = miss_val[snp][i];
      double x = 0;
      switch (type) {
        case A: x = (double)val; break;
        case H: x = (double)(val == 1); break;
        case D: x = (double)(val > 0); break;
        default: x = (double)(val == 2); break;
      }
      v[ml[i]] = x;
    }
  }
  /* src/data_model.cpp:78-103 */
  void sample_missing(const std::vector<int32_t>& model_inds, Rand& rng)
  {
    for (size_t snp = 0; snp < m_g; ++snp) {
      if (miss_val[snp].empty() || model_inds[snp] >= 0) continue;
      for (size_t i = 0; i < miss_val[snp].size(); ++i)
        miss_val[snp][i] = (char)sample_discrete_naive(data->miss_prior[snp].data(), 3, rng);
    }
  }
  void sample_missing_single(uint32_t snp, Rand& rng)
  {
    if (miss_val[snp].empty()) return;
    for (size_t i = 0; i < miss_val[snp].size(); ++i)
      miss_val[snp][i] = (char)sample_discrete_naive(data->miss_prior[snp].data(), 3, rng);
  }
  /* src/data_model.cpp:105-167 */
  void update_prexx_cov(size_t snp, double* pre_xx) const
  {
    if (miss_val[snp].empty()) return;
    double* xxloc = pre_xx;
    const std::vector<char>& mv = miss_val[snp];
    double sum_a_times_sum_h = 0.0;
    if (allow_types(AH)) sum_a_times_sum_h = pre_xx[0] * pre_xx[2];
    for (int t = 0; t < 4; ++t) {
      if (!allow_terms(t)) continue;
      double sg = 0.0, sg2 = 0.0, vg = 0.0;
      for (size_t i = 0; i < mv.size(); ++i) {
        char val = mv[i];
        switch (t) {
          case A: vg = (double)val; break;
          case H: vg = (double)(val == 1); break;
          case D: vg = (double)(val > 0); break;
          default: vg = (double)(val == 2); break;
        }
        sg += vg;
        sg2 += vg * vg;
      }
      double old_sum = *xxloc;
      *xxloc += sg;
      xxloc++;
      *xxloc += sg2 - sg * (old_sum * 2.0 + sg) / (double)n;
      xxloc++;
    }
    if (allow_types(AH)) {
      *xxloc += (sum_a_times_sum_h - pre_xx[0] * pre_xx[2]) / (double)n;
      for (size_t i = 0; i < mv.size(); ++i)
        if (mv[i] == 1) *xxloc += (double)mv[i];
    }
  }
};

/* ------------------------------------------------- precomputed covariances */
/* src/precomputed_snp_covariances.hpp:42-131 */
struct PreXX {
  int offset;
  int offset_type[4];
  std::vector<double> xx;
  explicit PreXX(const DataModel* dm)
  {
    bool ah = dm->allow_types(AH), a = dm->allow_types(A), h = dm->allow_types(H);
    offset = 2 * (int)dm->n_types + (ah ? 1 : 0) * (1 + ((a && h) ? -2 : 0) + ((a || h) ? 0 : 2));
    int i = 0;
    for (int j = 0; j < 4; ++j) offset_type[j] = dm->allow_terms(j) ? i++ : -1;
    size_t n = dm->n;
    xx.assign(dm->m_g * offset, 0.0);
    std::vector<double> x(n, 0.0), xah(n, 0.0);
    double* loc = xx.data();
    for (size_t s = 0; s < dm->m_g; ++s) {
      for (int t = 0; t < 4; ++t) {
        if (!dm->allow_terms(t)) continue;
        dm->get_genotypes(t, s, x.data());
        double xs = 0;
        for (size_t k = 0; k < n; ++k) xs += x[k];
        *loc++ = xs;
        *loc++ = ddot(n, x.data(), x.data()) - xs * xs / (double)n;
      }
      if (dm->allow_types(AH)) {
        dm->get_genotypes(A, s, x.data());
        dm->get_genotypes(H, s, xah.data());
        double as = 0, hs = 0;
        for (size_t k = 0; k < n; ++k) as += x[k];
        for (size_t k = 0; k < n; ++k) hs += xah[k];
        *loc++ = ddot(n, x.data(), xah.data()) - as * hs / (double)n;
      }
    }
  }
};

/* ------------------------------------------------------------------ prior */
struct Model;

/* src/prior.hpp:38-291, src/prior.cpp:30-141 */
struct Prior {
  double n_plus_nu, minus_n_plus_nu_2, nus2_plus_yy, mu_alpha;
  bool use_individual_tau2;
  size_t n, m_g, m_e;
  double g_a, g_b;
  std::vector<double> inv_tau2_e;
  double nu_sigma2, s2_sigma2;
  double nu_tau2[4], s2_tau2[4], nus2_tau2[4];
  double alpha_, alpha2_;
  double inv_tau2_alpha2[4];
  double types_prior[5], types_prior_sum;
  bool allow_types[5], allow_terms[5];

  Prior(const Data* data, const DataModel* dm, const double* tp, double e_q, double var_q,
        const std::vector<double>& ite, double nu_s, double s2_s, const double* nu_t,
        const double* s2_t, double mu_a, bool indiv)
  : n_plus_nu(data->n + nu_s), minus_n_plus_nu_2(-0.5 * n_plus_nu),
    nus2_plus_yy(nu_s * s2_s + data->yy), mu_alpha(mu_a), use_individual_tau2(indiv),
    n(data->n), m_g(data->m_g), m_e(data->m_e), inv_tau2_e(ite), nu_sigma2(nu_s),
    s2_sigma2(s2_s), alpha_(std::max(0.5, mu_a)), alpha2_(alpha_ * alpha_),
    types_prior_sum(0)
  {
    if (s2_sigma2 <= 0) throw std::runtime_error("Prior specification error: s2_sigma2 is not positive");
    if (nu_sigma2 < 0) throw std::runtime_error("Prior specification error: nu_sigma2 is negative.");
    solve_betadist_params(e_q, var_q);
    for (int i = 0; i < 5; ++i) {
      allow_types[i] = dm->allow_types(i);
      if (allow_types[i]) { types_prior[i] = tp[i]; types_prior_sum += tp[i]; }
      else types_prior[i] = NAN;
    }
    for (int i = 0; i < 4; ++i) {
      allow_terms[i] = dm->allow_terms(i);
      if (allow_terms[i]) {
        nu_tau2[i] = nu_t[i];
        s2_tau2[i] = s2_t[i];
        if (s2_tau2[i] <= 0) throw std::runtime_error("Prior specification error: s2_tau2 is not positive.");
        if (nu_tau2[i] <= 0) throw std::runtime_error("Prior specification error: nu_tau2 is not positive.");
        nus2_tau2[i] = nu_tau2[i] * s2_tau2[i];
        double tau2_init = nus2_tau2[i] / std::max(0.1, (nu_tau2[i] - 2));
        inv_tau2_alpha2[i] = 1.0 / (alpha2_ * tau2_init);
      } else {
        nu_tau2[i] = s2_tau2[i] = nus2_tau2[i] = inv_tau2_alpha2[i] = NAN;
      }
    }
    allow_terms[4] = false;
  }
  /* src/prior.hpp:273-290 */
  void solve_betadist_params(double e_q, double var_q)
  {
    if (m_g > 1) {
      double z = (var_q - e_q * (1 - e_q)) / ((m_g - 1) * e_q);
      g_a = (z - 1) / (1 - m_g * z / e_q);
      g_b = (m_g / e_q - 1) * g_a;
    } else {
      double z = e_q / (1 - e_q);
      g_b = z / var_q / pow(1 + z, 3) - 1 / (1 + z);
      g_a = z * g_b;
    }
    if (g_a <= 0 || g_b <= 0 || std::isnan(g_a) || std::isnan(g_b))
      throw std::runtime_error("Invalid a or b.");
  }
  /* src/prior.hpp:212-219 */
  double log_det_invQ_e() const
  {
    double log_sum_2 = 0.0;
    for (size_t i = 1; i < m_e; ++i) log_sum_2 += log(inv_tau2_e[i]);
    return log_sum_2;
  }
  /* src/prior.hpp:144-167 */
  double compute_log_change_on_add(const int* Ns, int nl, int type) const
  {
    return (log(g_a + nl) - log(g_b + m_g - nl - 1)) +
           (log(types_prior[type] + Ns[type]) - log(types_prior_sum + nl));
  }
  double compute_log_change_on_rem(const int* Ns, int nl, int type) const
  {
    return (log(g_b + m_g - nl) - log(g_a + nl - 1)) +
           (log(types_prior_sum + nl - 1) - log(types_prior[type] + Ns[type] - 1));
  }
  double compute_log_change_on_swi(const int* Ns, int ta, int tr) const
  {
    return (ta == tr) ? 0 : log(types_prior[ta] + Ns[ta]) - log(types_prior[tr] + Ns[tr] - 1);
  }
  /* src/prior.hpp:169-183 */
  double compute_log_model(const int* Ns) const
  {
    double lp = 0;
    int n_g = 0;
    for (int i = 0; i < 5; ++i) {
      if (allow_types[i]) {
        lp += std::lgamma(types_prior[i] + (double)Ns[i]);
        n_g += Ns[i];
      }
    }
    lp += std::lgamma(g_a + (double)n_g) + std::lgamma(g_b + (double)m_g - (double)n_g) -
          std::lgamma(types_prior_sum + (double)n_g);
    return lp;
  }
  double sample_single_inv_tau2_from_prior_times_alpha2(int type, Rand& rng) const
  {
    if (use_individual_tau2) return 1.0 / (alpha2_ * rng.rand_sinvchi2(nu_tau2[type], s2_tau2[type]));
    return inv_tau2_alpha2[type];
  }
  double e_g() const { return g_a / (g_a + g_b) * m_g; }
  void sample_alpha_and_tau2(Model* m, Rand& rng);
  double sample_alpha(Model* m, Rand& rng);
  void sample_tau2(Model* m, Rand& rng);
  void set_alpha(double val, Model* m);
};

/* ------------------------------------------------------------------ stats */
struct Stats {
  unsigned long n_add = 0, n_rem = 0, n_full = 0;
};

/* ------------------------------------------------------------------ model */
/* src/model.hpp:46-582.  Column-major storage with leading dimension cap. */
struct Model {
  const Data* data;
  const DataModel* dm;
  const Prior* prior;
  Stats* stats;
  size_t n, cap;
  std::vector<double> x;   /* n x cap */
  size_t xcols;
  std::vector<double> xx, l; /* cap x cap, upper */
  size_t llen;               /* active length of l (may differ from xcols transiently) */
  std::vector<double> xy, v, inv, beta, mu_beta, y_hat, y_hat_tmp_e, c_tmp, s_tmp;
  size_t vlen, blen;
  double sigma2, syx_plus_vs2, log_det_invQ, log_det_invQ_plus_xx;
  int Ns[5];
  bool mu_beta_computed;
  double log_likelihood_;
  std::vector<uint32_t> loci, x_ind_to_g_ind;
  std::vector<int32_t> model_inds;
  std::vector<unsigned char> type_inds;
  std::vector<int> x_types;
  std::vector<unsigned int> x_ind1, x_ind2;

  double& X(size_t i, size_t j) { return x[j * n + i]; }
  double& XX(size_t i, size_t j) { return xx[j * cap + i]; }
  double& L(size_t i, size_t j) { return l[j * cap + i]; }

  Model(const Data* d, const DataModel* m, const Prior* p, Stats* s, size_t cap_)
  : data(d), dm(m), prior(p), stats(s), n(d->n), cap(cap_), x(d->n * cap_, 0.0),
    xcols(d->m_e), xx(cap_ * cap_, 0.0), l(cap_ * cap_, 0.0), llen(d->m_e),
    xy(cap_, 0.0), v(cap_, 0.0), inv(cap_, 0.0), beta(cap_, 0.0), mu_beta(cap_, 0.0),
    y_hat(d->n, 0.0), y_hat_tmp_e(d->n, 0.0), c_tmp(cap_, 0.0), s_tmp(cap_, 0.0),
    vlen(d->m_e), blen(d->m_e), sigma2(0), syx_plus_vs2(0), log_det_invQ(0),
    log_det_invQ_plus_xx(0), mu_beta_computed(false), log_likelihood_(NAN),
    x_ind_to_g_ind(d->m_e, 0), model_inds(d->m_g + d->m_e, -1)
  {
    for (int i = 0; i < 5; ++i) Ns[i] = 0;
    if (d->m_e > cap) throw std::runtime_error("Not enough memory for initializing environmental data.");
    for (size_t j = 0; j < d->m_e; ++j)
      for (size_t i = 0; i < n; ++i) X(i, j) = d->e[j * n + i];
    cblas_dsyrk(CblasColMajor, CblasUpper, CblasTrans, (int)d->m_e, (int)n, 1.0, x.data(),
                (int)n, 0.0, xx.data(), (int)cap);
    cblas_dgemv(CblasColMajor, CblasTrans, (int)n, (int)d->m_e, 1.0, x.data(), (int)n,
                d->y.data(), 1, 0.0, xy.data(), 1);
    for (size_t i = 0; i < d->m_e; ++i) x_types.push_back(AH);
    for (size_t i = 0; i < d->m_e; ++i) inv[i] = p->inv_tau2_e[i];
    compute_log_likelihood();
  }

  /* src/model.hpp:115-162 (copies the active parts, as the reference does) */
  void copy_from(const Model& s)
  {
    xcols = s.xcols;
    std::memcpy(x.data(), s.x.data(), sizeof(double) * n * xcols);
    llen = s.llen;
    size_t xxl = s.xcols;
    for (size_t c = 0; c < xxl; ++c)
      for (size_t r = 0; r <= c; ++r) xx[c * cap + r] = s.xx[c * cap + r];
    for (size_t c = 0; c < s.llen; ++c)
      for (size_t r = 0; r <= c; ++r) l[c * cap + r] = s.l[c * cap + r];
    std::memcpy(xy.data(), s.xy.data(), sizeof(double) * s.xcols);
    vlen = s.vlen;
    std::memcpy(v.data(), s.v.data(), sizeof(double) * s.vlen);
    std::memcpy(inv.data(), s.inv.data(), sizeof(double) * s.xcols);
    blen = s.blen;
    std::memcpy(beta.data(), s.beta.data(), sizeof(double) * s.blen);
    std::memcpy(mu_beta.data(), s.mu_beta.data(), sizeof(double) * cap);
    sigma2 = s.sigma2;
    syx_plus_vs2 = s.syx_plus_vs2;
    log_det_invQ = s.log_det_invQ;
    log_det_invQ_plus_xx = s.log_det_invQ_plus_xx;
    std::memcpy(Ns, s.Ns, sizeof(Ns));
    mu_beta_computed = s.mu_beta_computed;
    log_likelihood_ = s.log_likelihood_;
    loci = s.loci;
    x_ind_to_g_ind = s.x_ind_to_g_ind;
    model_inds = s.model_inds;
    type_inds = s.type_inds;
    x_types = s.x_types;
    x_ind1 = s.x_ind1;
    x_ind2 = s.x_ind2;
  }

  size_t size() const { return loci.size(); }

  /* src/model.hpp:558-576 */
  double prepare_l_chol_and_get_det_invQ()
  {
    llen = xcols;
    for (size_t c = 0; c < xcols; ++c)
      for (size_t r = 0; r <= c; ++r) L(r, c) = XX(r, c);
    double log_sum_2 = 0;
    L(0, 0) += inv[0];
    for (size_t i = 1; i < llen; ++i) {
      L(i, i) += inv[i];
      log_sum_2 += log(inv[i]);
    }
    return 0.5 * log_sum_2;
  }

  /* src/model.hpp:199-237 */
  void compute_log_likelihood()
  {
    if (xcols < 1) { log_likelihood_ = NAN; return; }
    stats->n_full++;
    log_det_invQ = prepare_l_chol_and_get_det_invQ();
    char uplo = 'U';
    int info = -1, len = (int)llen, ld = (int)cap;
    dpotrf_(&uplo, &len, l.data(), &ld, &info);
    if (info != 0) {
      log_likelihood_ = -INFINITY;
      syx_plus_vs2 = INFINITY;
      mu_beta_computed = false;
      return;
    }
    vlen = xcols;
    for (size_t i = 0; i < xcols; ++i) v[i] = xy[i];
    cblas_dtrsv(CblasColMajor, CblasUpper, CblasTrans, CblasNonUnit, (int)llen, l.data(),
                (int)cap, v.data(), 1);
    syx_plus_vs2 = prior->nus2_plus_yy - ddot(vlen, v.data(), v.data());
    log_det_invQ_plus_xx = 0;
    for (size_t i = 0; i < llen; ++i) log_det_invQ_plus_xx += log(L(i, i));
    log_likelihood_ = log_det_invQ - log_det_invQ_plus_xx + prior->minus_n_plus_nu_2 * log(syx_plus_vs2);
    mu_beta_computed = false;
  }

  /* src/model.hpp:239-268 */
  void add_term(uint32_t ind, int t_ind, const double* inv_vals, bool update = true)
  {
    int type = dm->types[t_ind];
    bool is_ah = (type == AH);
    size_t model_ind = loci.size();
    if (xcols + 1 + (size_t)is_ah > cap) throw std::runtime_error("Not enough memory for adding term.");
    loci.push_back(ind);
    ++Ns[type];
    type_inds.push_back((unsigned char)t_ind);
    model_inds[ind] = (int32_t)model_ind;
    mu_beta_computed = false;
    if (is_ah) {
      update_likelihood_on_add(ind, model_ind, A, false, inv_vals[0], update);
      if (std::isfinite(syx_plus_vs2))
        update_likelihood_on_add(ind, model_ind, H, true, inv_vals[1], update);
    } else {
      update_likelihood_on_add(ind, model_ind, type, false, inv_vals[0], update);
    }
  }

  /* src/model.hpp:270-312 */
  void remove_term(int model_ind, bool update = true)
  {
    uint32_t ind = loci[model_ind];
    int type = dm->types[type_inds[model_ind]];
    unsigned int xi1 = x_ind1[model_ind], xi2 = x_ind2[model_ind];
    model_inds[ind] = -1;
    --Ns[type];
    loci.erase(loci.begin() + model_ind);
    type_inds.erase(type_inds.begin() + model_ind);
    x_ind1.erase(x_ind1.begin() + model_ind);
    x_ind2.erase(x_ind2.begin() + model_ind);
    int xmove = (type == AH) ? 2 : 1;
    for (size_t i = model_ind; i < loci.size(); ++i) {
      x_ind1[i] -= xmove;
      x_ind2[i] -= xmove;
      model_inds[loci[i]]--;
    }
    if (type == AH) {
      if (xi1 > xi2) {
        update_likelihood_on_remove(xi1, update);
        update_likelihood_on_remove(xi2, update);
      } else {
        update_likelihood_on_remove(xi2, update);
        update_likelihood_on_remove(xi1, update);
      }
    } else {
      update_likelihood_on_remove(xi1, update);
    }
    mu_beta_computed = false;
  }

  /* src/model.hpp:314-324 */
  void compute_mu_beta()
  {
    if (mu_beta_computed) return;
    for (size_t i = 0; i < vlen; ++i) mu_beta[i] = v[i];
    cblas_dtrsv(CblasColMajor, CblasUpper, CblasNoTrans, CblasNonUnit, (int)llen, l.data(),
                (int)cap, mu_beta.data(), 1);
    mu_beta_computed = true;
  }

  /* src/model.hpp:326-342, src/rand.hpp:144-168 */
  void sample_beta_sigma2(Rand& rng)
  {
    sigma2 = rng.rand_sinvchi2(syx_plus_vs2 / prior->n_plus_nu);
    compute_mu_beta();
    blen = vlen;
    for (size_t i = 0; i < blen; ++i) beta[i] = rng.rand_normal();
    cblas_dtrsv(CblasColMajor, CblasUpper, CblasNoTrans, CblasNonUnit, (int)llen, l.data(),
                (int)cap, beta.data(), 1);
    double scale = sqrt(sigma2);
    for (size_t i = 0; i < blen; ++i) beta[i] = scale * beta[i] + mu_beta[i];
  }

  /* src/model.hpp:345-392 */
  void compute_pve(double* pves)
  {
    size_t m_e = dm->m_e;
    bool ce = (m_e > 1);
    if (ce) {
      cblas_dgemv(CblasColMajor, CblasNoTrans, (int)n, (int)m_e, 1.0, x.data(), (int)n,
                  beta.data(), 1, 0.0, y_hat_tmp_e.data(), 1);
      pves[2] = var(y_hat_tmp_e);
    } else {
      pves[2] = 0.0;
      for (size_t i = 0; i < n; ++i) y_hat_tmp_e[i] = beta[0];
    }
    bool cg = (loci.size() > 0);
    if (cg) {
      cblas_dgemv(CblasColMajor, CblasNoTrans, (int)n, (int)(xcols - m_e), 1.0, x.data() + m_e * n,
                  (int)n, beta.data() + m_e, 1, 0.0, y_hat.data(), 1);
      pves[1] = var(y_hat);
    } else {
      pves[1] = 0.0;
    }
    if (ce || cg) {
      for (size_t i = 0; i < n; ++i) y_hat[i] += y_hat_tmp_e[i];
      if (!ce) pves[0] = pves[1];
      else if (!cg) pves[0] = pves[2];
      else pves[0] = var(y_hat);
    } else {
      for (size_t i = 0; i < n; ++i) y_hat[i] = y_hat_tmp_e[i];
      pves[0] = pves[1] = pves[2] = 0;
      return;
    }
    double z = pves[0] + sigma2;
    pves[0] /= z;
    pves[1] /= z;
    pves[2] /= z;
  }

  static double var(const std::vector<double>& a)
  {
    double sq = 0, s = 0;
    size_t len = a.size();
    for (size_t i = 0; i < len; ++i) { sq += a[i] * a[i]; s += a[i]; }
    return (sq - s * s / len) / (len - 1);
  }

  /* src/model.hpp:432-506, src/symmmatrix.cpp:144-164 */
  void update_likelihood_on_add(uint32_t ind, size_t model_ind, int type, bool is_x_ind2,
                                double inv_val, bool update)
  {
    size_t col = xcols;
    if (is_x_ind2) x_ind2[model_ind] = (unsigned)col;
    else { x_ind1.push_back((unsigned)col); x_ind2.push_back(0); }
    x_ind_to_g_ind.push_back(ind);
    x_types.push_back(type);
    xcols = col + 1;
    double* xcol = &x[col * n];
    dm->get_genotypes(type, ind, xcol);
    xy[col] = ddot(n, xcol, data->y.data());
    inv[col] = inv_val;
    double* xxcol = &xx[col * cap];
    cblas_dgemv(CblasColMajor, CblasTrans, (int)n, (int)(col + 1), 1.0, x.data(), (int)n,
                xcol, 1, 0.0, xxcol, 1);
    if (!update) { llen = col + 1; vlen = col + 1; return; }
    stats->n_add++;
    /* cholesky_update */
    double* lcol = &l[col * cap];
    for (size_t i = 0; i <= col; ++i) lcol[i] = xxcol[i];
    cblas_dtrsv(CblasColMajor, CblasUpper, CblasTrans, CblasNonUnit, (int)col, l.data(),
                (int)cap, lcol, 1);
    double lmm2 = xxcol[col] + inv_val - ddot(col, lcol, lcol);
    llen = col + 1;
    if (lmm2 <= 0) {
      log_likelihood_ = -INFINITY;
      syx_plus_vs2 = INFINITY;
      mu_beta_computed = false;
      vlen = col + 1;
      return;
    }
    L(col, col) = sqrt(lmm2);
    double vm2 = xy[col] - ddot(col, lcol, v.data());
    vlen = col + 1;
    v[col] = vm2 / L(col, col);
    vm2 = v[col] * v[col];
    syx_plus_vs2 = syx_plus_vs2 - vm2;
    log_det_invQ += 0.5 * log(inv_val);
    log_det_invQ_plus_xx += log(L(col, col));
    log_likelihood_ = log_det_invQ - log_det_invQ_plus_xx + prior->minus_n_plus_nu_2 * log(syx_plus_vs2);
  }

  /* src/model.hpp:508-556, src/symmmatrix.cpp:126-195 */
  void update_likelihood_on_remove(unsigned int x_ind, bool update)
  {
    /* x.remove_column */
    std::memmove(&x[x_ind * n], &x[(x_ind + 1) * n], (xcols - x_ind - 1) * n * sizeof(double));
    x_ind_to_g_ind.erase(x_ind_to_g_ind.begin() + x_ind);
    std::memmove(&xy[x_ind], &xy[x_ind + 1], (xcols - x_ind - 1) * sizeof(double));
    /* xx.remove_colrow */
    size_t len = xcols;
    for (size_t i = x_ind; i < len - 1; ++i)
      for (size_t j = 0; j <= i; ++j)
        XX(j, i) = (j < x_ind) ? XX(j, i + 1) : XX(j + 1, i + 1);
    x_types.erase(x_types.begin() + x_ind);
    double inv_val = inv[x_ind];
    std::memmove(&inv[x_ind], &inv[x_ind + 1], (xcols - x_ind - 1) * sizeof(double));
    xcols = len - 1;
    if (update) {
      stats->n_rem++;
      if (x_ind == xcols) {
        log_det_invQ_plus_xx -= log(L(x_ind, x_ind));
        syx_plus_vs2 += v[x_ind] * v[x_ind];
        llen = xcols;
        vlen = xcols;
      } else {
        int col_rem_f = (int)x_ind + 1, ld = (int)cap, m = (int)llen, z0 = 0, job = 2;
        dchex_(l.data(), &ld, &m, &col_rem_f, &m, nullptr, &z0, &z0, c_tmp.data(), s_tmp.data(), &job);
        llen = (size_t)m - 1;
        for (size_t i = x_ind; i < llen; ++i) {
          if (L(i, i) < 0)
            for (size_t j = i; j < llen; ++j) L(i, j) *= -1;
        }
        vlen = xcols;
        for (size_t i = 0; i < vlen; ++i) v[i] = xy[i];
        cblas_dtrsv(CblasColMajor, CblasUpper, CblasTrans, CblasNonUnit, (int)llen, l.data(),
                    (int)cap, v.data(), 1);
        log_det_invQ_plus_xx = 0;
        for (size_t i = 0; i < llen; ++i) log_det_invQ_plus_xx += log(L(i, i));
        syx_plus_vs2 = prior->nus2_plus_yy - ddot(vlen, v.data(), v.data());
      }
      log_det_invQ -= 0.5 * log(inv_val);
      log_likelihood_ = log_det_invQ - log_det_invQ_plus_xx + prior->minus_n_plus_nu_2 * log(syx_plus_vs2);
    } else {
      llen = xcols;
      vlen = xcols;
    }
  }

  /* src/symmmatrix.cpp:220-264: swap columns col and col + 1 of the upper
     Cholesky factor (length llen, leading dimension cap) and restore it with
     one Givens rotation; rotate v alongside */
  void cholesky_swapadj(size_t col, std::vector<double>* vv)
  {
    double* col1 = l.data() + col * cap;
    double* col2 = col1 + cap;
    for (size_t i = 0; i < col + 2; ++i) std::swap(*col1++, *col2++);
    *(--col2) = 0.0;
    col1 = l.data() + col * cap + col;
    col2 = col1 + 1;
    double c, sn;
    cblas_drotg(col1, col2, &c, &sn);
    if (*col1 < 0) {
      *col1 *= -1.0;
      sn *= -1.0;
      c *= -1.0;
    }
    double tmp;
    for (size_t i = col + 1; i < llen; ++i) {
      col1 += cap;
      col2 = col1 + 1;
      tmp = *col1 * sn - *col2 * c;
      *col1 = *col2 * sn + *col1 * c;
      *col2 = tmp;
    }
    if (vv) {
      col1 = &(*vv)[col];
      col2 = &(*vv)[col + 1];
      tmp = *col1 * sn - *col2 * c;
      *col1 = *col2 * sn + *col1 * c;
      *col2 = tmp;
    }
  }
};

/* src/model.hpp:585-844: the last n terms of a model, whose 2^n sub-models
   are visited by adding terms and moving them left (delayed rejection) */
struct ExhModel : Model {
  size_t model_size_ = 0, const_loci_ = 0, v_size_ = 0;
  double log_model_prior_ = 0.0;

  ExhModel(const Data* d, const DataModel* m, const Prior* p, Stats* s, size_t cap_) : Model(d, m, p, s, cap_) {}

  double log_prob() const { return log_likelihood_ + log_model_prior_; }

  double update_to_model(const Model& src, size_t const_loci)
  {
    llen = src.llen;
    for (size_t c = 0; c < src.llen; ++c)
      for (size_t r = 0; r <= c; ++r) l[c * cap + r] = src.l[c * cap + r];
    std::memcpy(xy.data(), src.xy.data(), sizeof(double) * src.xcols);
    vlen = src.vlen;
    std::memcpy(v.data(), src.v.data(), sizeof(double) * src.vlen);
    std::memcpy(inv.data(), src.inv.data(), sizeof(double) * src.xcols);
    type_inds = src.type_inds;
    x_types = src.x_types;
    x_ind1 = src.x_ind1;
    x_ind2 = src.x_ind2;
    const_loci_ = const_loci;
    model_size_ = const_loci_;
    if (model_size_ > 0) {
      if (AH == dm->types[type_inds[model_size_ - 1]]) v_size_ = x_ind2[model_size_ - 1] + 1;
      else v_size_ = x_ind1[model_size_ - 1] + 1;
    } else {
      v_size_ = dm->m_e;
    }
    syx_plus_vs2 = prior->nus2_plus_yy - ddot(v_size_, v.data(), v.data());
    log_det_invQ_plus_xx = 0;
    for (size_t i = 0; i < v_size_; i++) log_det_invQ_plus_xx += log(L(i, i));
    log_det_invQ = prior->log_det_invQ_e();
    for (size_t i = dm->m_e; i < v_size_; ++i) log_det_invQ += log(inv[i]);
    log_det_invQ *= 0.5;
    log_likelihood_ = log_det_invQ - log_det_invQ_plus_xx + prior->minus_n_plus_nu_2 * log(syx_plus_vs2);
    log_model_prior_ = 0.0;
    for (int i = 0; i < 5; ++i) Ns[i] = 0;
    for (size_t i = 0; i < model_size_; ++i) ++Ns[dm->types[type_inds[i]]];
    return log_likelihood_ + log_model_prior_;
  }

  double update_on_add()
  {
    int type = dm->types[type_inds[model_size_]];
    syx_plus_vs2 -= v[v_size_] * v[v_size_];
    log_det_invQ += 0.5 * log(inv[v_size_]);
    log_det_invQ_plus_xx += log(L(v_size_, v_size_));
    ++v_size_;
    if (AH == type) {
      syx_plus_vs2 -= v[v_size_] * v[v_size_];
      log_det_invQ += 0.5 * log(inv[v_size_]);
      log_det_invQ_plus_xx += log(L(v_size_, v_size_));
      ++v_size_;
    }
    log_likelihood_ = log_det_invQ - log_det_invQ_plus_xx + prior->minus_n_plus_nu_2 * log(syx_plus_vs2);
    log_model_prior_ += prior->compute_log_change_on_add(Ns, (int)model_size_, type);
    ++Ns[type];
    ++model_size_;
    return log_likelihood_ + log_model_prior_;
  }

  double update_on_moveleft()
  {
    --model_size_;
    size_t ind_keep = model_size_;
    size_t ind_rem = model_size_ - 1;
    int type_keep = dm->types[type_inds[ind_keep]];
    int type_rem = dm->types[type_inds[ind_rem]];
    --v_size_;
    syx_plus_vs2 += v[v_size_] * v[v_size_];
    log_det_invQ_plus_xx -= log(L(v_size_, v_size_));
    if (AH == type_keep) {
      --v_size_;
      syx_plus_vs2 += v[v_size_] * v[v_size_];
      log_det_invQ_plus_xx -= log(L(v_size_, v_size_));
    }
    --v_size_;
    syx_plus_vs2 += v[v_size_] * v[v_size_];
    log_det_invQ -= 0.5 * log(inv[v_size_]);
    log_det_invQ_plus_xx -= log(L(v_size_, v_size_));
    if (AH == type_rem) {
      --v_size_;
      syx_plus_vs2 += v[v_size_] * v[v_size_];
      log_det_invQ -= 0.5 * log(inv[v_size_]);
      log_det_invQ_plus_xx -= log(L(v_size_, v_size_));
    }
    std::swap(type_inds[ind_keep], type_inds[ind_rem]);
    if (AH == type_rem) {
      if (AH == type_keep) {
        size_t swap_ind = x_ind2[ind_rem];
        cholesky_swapadj(swap_ind, &v);
        ++swap_ind;
        cholesky_swapadj(swap_ind, &v);
        swap_ind -= 2;
        cholesky_swapadj(swap_ind, &v);
        ++swap_ind;
        cholesky_swapadj(swap_ind, &v);
        std::swap(xy[x_ind1[ind_keep]], xy[x_ind2[ind_rem]]);
        std::swap(xy[x_ind1[ind_keep]], xy[x_ind2[ind_keep]]);
        std::swap(xy[x_ind1[ind_rem]], xy[x_ind2[ind_rem]]);
        std::swap(xy[x_ind1[ind_keep]], xy[x_ind2[ind_rem]]);
        std::swap(inv[x_ind1[ind_keep]], inv[x_ind2[ind_rem]]);
        std::swap(inv[x_ind1[ind_keep]], inv[x_ind2[ind_keep]]);
        std::swap(inv[x_ind1[ind_rem]], inv[x_ind2[ind_rem]]);
        std::swap(inv[x_ind1[ind_keep]], inv[x_ind2[ind_rem]]);
      } else {
        size_t swap_ind = x_ind2[ind_rem];
        cholesky_swapadj(swap_ind, &v);
        --swap_ind;
        cholesky_swapadj(swap_ind, &v);
        std::swap(xy[x_ind2[ind_rem]], xy[x_ind1[ind_keep]]);
        std::swap(xy[x_ind1[ind_rem]], xy[x_ind2[ind_rem]]);
        std::swap(inv[x_ind2[ind_rem]], inv[x_ind1[ind_keep]]);
        std::swap(inv[x_ind1[ind_rem]], inv[x_ind2[ind_rem]]);
        std::swap(x_types[x_ind2[ind_rem]], x_types[x_ind1[ind_keep]]);
        std::swap(x_types[x_ind1[ind_rem]], x_types[x_ind2[ind_rem]]);
        x_ind2[ind_keep] = x_ind1[ind_keep];
        --x_ind1[ind_keep];
      }
    } else {
      if (AH == type_keep) {
        size_t swap_ind = x_ind1[ind_rem];
        cholesky_swapadj(swap_ind, &v);
        ++swap_ind;
        cholesky_swapadj(swap_ind, &v);
        std::swap(xy[x_ind1[ind_rem]], xy[x_ind1[ind_keep]]);
        std::swap(xy[x_ind1[ind_keep]], xy[x_ind2[ind_keep]]);
        std::swap(inv[x_ind1[ind_rem]], inv[x_ind1[ind_keep]]);
        std::swap(inv[x_ind1[ind_keep]], inv[x_ind2[ind_keep]]);
        std::swap(x_types[x_ind1[ind_rem]], x_types[x_ind1[ind_keep]]);
        std::swap(x_types[x_ind1[ind_keep]], x_types[x_ind2[ind_keep]]);
        x_ind2[ind_rem] = x_ind1[ind_keep];
        x_ind1[ind_keep] = x_ind2[ind_keep];
      } else {
        size_t swap_ind = x_ind1[ind_rem];
        cholesky_swapadj(swap_ind, &v);
        std::swap(xy[x_ind1[ind_keep]], xy[x_ind1[ind_rem]]);
        std::swap(inv[x_ind1[ind_keep]], inv[x_ind1[ind_rem]]);
        std::swap(x_types[x_ind1[ind_keep]], x_types[x_ind1[ind_rem]]);
      }
    }
    syx_plus_vs2 -= v[v_size_] * v[v_size_];
    log_det_invQ_plus_xx += log(L(v_size_, v_size_));
    ++v_size_;
    if (AH == type_keep) {
      syx_plus_vs2 -= v[v_size_] * v[v_size_];
      log_det_invQ_plus_xx += log(L(v_size_, v_size_));
      ++v_size_;
    }
    log_likelihood_ = log_det_invQ - log_det_invQ_plus_xx + prior->minus_n_plus_nu_2 * log(syx_plus_vs2);
    log_model_prior_ += prior->compute_log_change_on_rem(Ns, (int)model_size_ + 1, type_rem);
    --Ns[type_rem];
    return log_likelihood_ + log_model_prior_;
  }

  double update_on_twonewswap()
  {
    update_on_add();
    update_on_add();
    return update_on_moveleft();
  }
};

/* src/sampler.cpp:882-978: the log probabilities of all 2^n_inds sub-models
   of the exhaustive model's last n_inds terms, by adds and left moves */
static void compute_exhaustive_modelset(size_t n_inds, ExhModel* exhmodel, double* log_model_probabilities,
                                        double& max_log_model)
{
  size_t nmodels = 0, tmp;
  size_t cmodel_binary = 0;
  int model_size = 0;
  std::vector<size_t> cmodel_inds(n_inds);
  for (size_t i = 0; i < n_inds; ++i) cmodel_inds[i] = i;
  log_model_probabilities[cmodel_binary] = exhmodel->log_prob();
  max_log_model = log_model_probabilities[cmodel_binary];
  for (size_t i = 0; i < n_inds; ++i) {
    ++model_size;
    if (i > 1) {
      ++model_size;
      exhmodel->update_on_add();
    }
    cmodel_binary = (size_t)std::pow(2, model_size) - 1;
    log_model_probabilities[cmodel_binary] = exhmodel->update_on_add();
    if (log_model_probabilities[cmodel_binary] > max_log_model) max_log_model = log_model_probabilities[cmodel_binary];
    for (size_t j = 0; j < i; ++j) {
      --model_size;
      tmp = cmodel_inds[model_size - 1];
      cmodel_inds[model_size - 1] = cmodel_inds[model_size];
      cmodel_inds[model_size] = tmp;
      cmodel_binary &= ~(1 << tmp);
      log_model_probabilities[cmodel_binary] = exhmodel->update_on_moveleft();
      if (log_model_probabilities[cmodel_binary] > max_log_model) max_log_model = log_model_probabilities[cmodel_binary];
    }
    nmodels = (size_t)std::pow(2, i) - i - 1;
    size_t j = 0;
    size_t K, nK = 0;
    char do_lefts = 0;
    while (j < nmodels) {
      if (do_lefts < 2) {
        ++model_size;
        tmp = cmodel_inds[model_size];
        cmodel_inds[model_size] = cmodel_inds[model_size - 1];
        cmodel_inds[model_size - 1] = tmp;
        cmodel_binary |= (1 << tmp);
        log_model_probabilities[cmodel_binary] = exhmodel->update_on_twonewswap();
        if (log_model_probabilities[cmodel_binary] > max_log_model)
          max_log_model = log_model_probabilities[cmodel_binary];
        ++j;
        ++do_lefts;
      } else {
        ++nK;
        K = 0;
        while (((nK >> K) & 1) == 0) K++;
        for (size_t k = 0; k <= K; ++k) {
          --model_size;
          tmp = cmodel_inds[model_size - 1];
          cmodel_inds[model_size - 1] = cmodel_inds[model_size];
          cmodel_inds[model_size] = tmp;
          cmodel_binary &= ~(1 << tmp);
          log_model_probabilities[cmodel_binary] = exhmodel->update_on_moveleft();
          if (log_model_probabilities[cmodel_binary] > max_log_model)
            max_log_model = log_model_probabilities[cmodel_binary];
          ++j;
        }
        do_lefts = 0;
      }
    }
  }
}

/* src/sampler.cpp:980-1049: adds the log proposal probability of reaching
   each sub-model from the "empty" one (adds in order, removals in reverse) */
static void compute_proposal_probs_for_exh_modelset(bool use_types, int n_inds,
                                                    const unsigned char* bit_to_normalized_order,
                                                    const double* q_add, const double* q_rem, double z_add,
                                                    double z_rem, size_t const_loci, size_t m_g,
                                                    const double* log_q_add_types, double* log_prop_probs)
{
  std::vector<char> isadd(n_inds);
  unsigned long nmodels = (unsigned long)std::pow(2, n_inds);
  for (unsigned long i = 0; i < nmodels; ++i) {
    size_t max_adds = m_g - const_loci;
    size_t max_rems = const_loci;
    double z_a = z_add;
    double z_r = z_rem;
    for (int j = 0; j < n_inds; ++j) {
      unsigned char bit = (i >> j) & 1;
      unsigned char nind = bit_to_normalized_order[j];
      if (bit) {
        isadd[nind] = false;
        z_a -= q_add[nind];
        z_r += q_rem[nind];
        ++max_rems;
        --max_adds;
      } else {
        isadd[nind] = true;
      }
    }
    int last_rem_pos = n_inds - 1;
    for (int j = 0; j < n_inds; ++j) {
      if (max_adds > 0 && max_rems > 0) log_prop_probs[i] += kLogHalf;
      if (isadd[j]) {
        --max_adds;
        log_prop_probs[i] += log(q_add[j]) - log(z_a);
        z_a -= q_add[j];
        if (use_types) log_prop_probs[i] += log_q_add_types[j];
      } else {
        --max_rems;
        while (isadd[last_rem_pos]) --last_rem_pos;
        log_prop_probs[i] += log(q_rem[last_rem_pos]) - log(z_r);
        z_r -= q_rem[last_rem_pos];
        --last_rem_pos;
      }
    }
  }
}

/* src/prior.cpp:30-69 */
double Prior::sample_alpha(Model* model, Rand& rng)
{
  size_t nterms = model->blen - m_e;
  double a = alpha_;
  do {
    if (nterms > 0) {
      if ((a <= 0.0) || log(rng.rand_01()) <= -2.0 * mu_alpha * a) a = -a;
      std::vector<double> xb(n), eb(n);
      cblas_dgemv(CblasColMajor, CblasNoTrans, (int)n, (int)nterms, 1.0,
                  model->x.data() + m_e * n, (int)n, model->beta.data() + m_e, 1, 0.0, xb.data(), 1);
      cblas_dgemv(CblasColMajor, CblasNoTrans, (int)n, (int)m_e, 1.0, model->x.data(), (int)n,
                  model->beta.data(), 1, 0.0, eb.data(), 1);
      for (size_t i = 0; i < n; ++i) eb[i] -= model->data->y[i];
      double alpha_sigma2 = a * model->sigma2;
      double var = 1.0 / (1.0 + ddot(n, xb.data(), xb.data()) / (a * alpha_sigma2));
      double mu = var * (mu_alpha - ddot(n, eb.data(), xb.data()) / alpha_sigma2);
      a = sqrt(var) * rng.rand_normal() + mu;
    } else {
      a = rng.rand_normal() + mu_alpha;
    }
  } while (a == 0 || a * a == 0);
  model->mu_beta_computed = false;
  return a;
}

/* src/prior.cpp:71-114 */
void Prior::sample_tau2(Model* model, Rand& rng)
{
  double alpha2_sigma2 = alpha2_ * model->sigma2;
  if (use_individual_tau2) {
    for (size_t i = m_e; i < model->blen; ++i) {
      int t = model->x_types[i];
      double nu = nu_tau2[t] + 1.0;
      double s2 = (nus2_tau2[t] + model->beta[i] * model->beta[i] / alpha2_sigma2) / nu;
      model->inv[i] = 1.0 / (alpha2_ * rng.rand_sinvchi2(nu, s2));
    }
  } else {
    size_t m = model->blen;
    double b2s[4] = {0, 0, 0, 0};
    size_t mt[4] = {0, 0, 0, 0};
    for (size_t i = m_e; i < m; ++i) {
      b2s[model->x_types[i]] += model->beta[i] * model->beta[i];
      ++mt[model->x_types[i]];
    }
    for (int t = 0; t < 4; ++t) {
      if (!allow_terms[t]) continue;
      double nu = nu_tau2[t] + mt[t];
      double s2 = (nus2_tau2[t] + b2s[t] / alpha2_sigma2) / nu;
      inv_tau2_alpha2[t] = 1.0 / (alpha2_ * rng.rand_sinvchi2(nu, s2));
    }
    for (size_t i = m_e; i < m; ++i) model->inv[i] = inv_tau2_alpha2[model->x_types[i]];
  }
  model->mu_beta_computed = false;
}

/* src/prior.cpp:116-141 */
void Prior::set_alpha(double val, Model* model)
{
  double old_alpha2 = alpha2_;
  alpha_ = val;
  alpha2_ = alpha_ * alpha_;
  if (use_individual_tau2) {
    for (size_t i = m_e; i < model->blen; ++i) model->inv[i] = model->inv[i] * old_alpha2 / alpha2_;
  } else {
    for (int t = 0; t < 4; ++t)
      if (allow_terms[t]) inv_tau2_alpha2[t] = inv_tau2_alpha2[t] * old_alpha2 / alpha2_;
    for (size_t i = m_e; i < model->blen; ++i) model->inv[i] = inv_tau2_alpha2[model->x_types[i]];
  }
}

void Prior::sample_alpha_and_tau2(Model* m, Rand& rng)
{
  sample_tau2(m, rng);
  set_alpha(sample_alpha(m, rng), m);
}

/* ----------------------------------------------- discrete distribution */
/* src/discrete_distribution.hpp:64-330: threaded binary tree in heap order;
 * node value = own weight + weight of the left subtree. */
struct DD {
  std::vector<int> parent, left, right, upright;
  std::vector<double> value;
  std::vector<unsigned char> zero;
  const double* w;
  size_t size;
  double total_w;
  int rightmost;
  Rand* rng;

  DD(const double* weights, size_t n, Rand* r) : w(weights), size(n), total_w(0), rng(r)
  {
    parent.assign(n, -1); left.assign(n, -1); right.assign(n, -1); upright.assign(n, -1);
    value.assign(n, 0.0); zero.assign(n, 0);
    value[0] = w[0];
    for (size_t ind = 1; ind < n; ++ind) {
      int pind = (int)((ind - 1) / 2);
      parent[ind] = pind;
      if (ind % 2 == 0) {
        right[pind] = (int)ind;
        int tmp = pind;
        while (parent[tmp] >= 0) {
          if (left[parent[tmp]] == tmp) { upright[ind] = parent[tmp]; break; }
          tmp = parent[tmp];
        }
      } else {
        left[pind] = (int)ind;
        upright[ind] = pind;
      }
    }
    rightmost = 0;
    while (right[rightmost] >= 0) rightmost = right[rightmost];
    update_tree_weights();
  }
  void update_weights(const double* weights) { w = weights; update_tree_weights(); }
  /* src/discrete_distribution.hpp:263-314 */
  void update_tree_weights()
  {
    int node = 0;
    bool went_upright = false;
    while (node != rightmost) {
      if (went_upright) {
        went_upright = false;
        if (right[node] >= 0) {
          node = right[node];
        } else {
          int tmp = node;
          node = upright[node];
          while (tmp != node) { value[node] += value[tmp]; tmp = parent[tmp]; }
          went_upright = true;
        }
      } else {
        value[node] = zero[node] ? 0.0 : w[node];
        if (left[node] >= 0) {
          node = left[node];
        } else {
          int tmp = node;
          node = upright[node];
          while (tmp != node) { value[node] += value[tmp]; tmp = parent[tmp]; }
          went_upright = true;
        }
      }
    }
    value[node] = zero[node] ? 0.0 : w[node];
    if (left[node] >= 0) {
      int lc = left[node];
      value[lc] = zero[lc] ? 0.0 : w[lc];
      value[node] += value[lc];
    }
    compute_total_w();
  }
  void compute_total_w()
  {
    int node = 0;
    total_w = value[node];
    while (right[node] >= 0) { node = right[node]; total_w += value[node]; }
  }
  /* src/discrete_distribution.hpp:125-153 */
  size_t sample()
  {
    double r = rng->rand_01() * total_w;
    double carry = 0.0;
    int node = 0;
    while (left[node] >= 0) {
      if (r < value[node] + carry) {
        node = left[node];
      } else {
        carry += value[node];
        if (right[node] >= 0) node = right[node];
        else return (size_t)upright[node];
      }
    }
    if (r < value[node] + carry) return (size_t)node;
    return (size_t)upright[node];
  }
  /* src/discrete_distribution.hpp:156-183 */
  void adddate(size_t ind)
  {
    int node = (int)ind;
    zero[node] = 1;
    if (left[node] >= 0) {
      value[node] = value[left[node]];
      int t = right[left[node]];
      while (t >= 0) { value[node] += value[t]; t = right[t]; }
    } else {
      value[node] = 0.0;
    }
    while (upright[node] >= 0) {
      node = upright[node];
      value[node] = (zero[node] ? 0.0 : w[node]) + value[left[node]];
      int t = right[left[node]];
      while (t >= 0) { value[node] += value[t]; t = right[t]; }
    }
    compute_total_w();
  }
  /* src/discrete_distribution.hpp:186-199 */
  void remdate(size_t ind)
  {
    double val = w[ind];
    int node = (int)ind;
    zero[node] = 0;
    value[node] += val;
    while (upright[node] >= 0) { node = upright[node]; value[node] += val; }
    total_w += val;
  }
};

/* --------------------------------------------------------------- sampler */
struct Trace {
  std::vector<uint8_t> jump, mtype, msize, types;
  std::vector<uint32_t> msz, loci;
  std::vector<double> ll, lp, s2, alpha, pve, beta;
  void clear()
  {
    jump.clear(); mtype.clear(); msize.clear(); types.clear(); msz.clear(); loci.clear();
    ll.clear(); lp.clear(); s2.clear(); alpha.clear(); pve.clear(); beta.clear();
  }
};

/* src/sampler.hpp:103-1776, src/sampler.cpp:32-880 */
struct Sampler {
  const bmg_options& o;
  const Data* data;
  const PreXX* pre;
  size_t n_iter, do_n_iter, n_accepted, n_rao, n_rao_burnin, n_sample_tau2;
  bool flat_proposal_dist, adaptation, save_beta;
  size_t thin;
  size_t m_g, n_types;
  bool use_types;
  uint32_t seed;
  Stats stats;
  Rand rng;
  DataModel* dm;
  Prior* prior;
  Model* cur;
  Model* nm;
  std::vector<double> p_proposal, p_proposal_types;
  size_t p_proposal_n;
  std::vector<double> p_rao, p_rao_types;
  int p_rao_n;
  double p_moves[7], p_moves_cumsum[7];
  std::vector<double> q_add, q_rem, p_r, p_r_types, q_add_types, q_p_add_types;
  double q_add_min, q_rem_min;
  double q_p_add_types_tmp[5];
  DD* dd_add;
  DD* dd_rem;
  unsigned char max_move_size;
  size_t max_nbh;
  double p_move_size, p_move_size_nbs, p_move_size_nbc;
  bool adapt_p_move_size;
  std::vector<double> q_p_move_size, q_p_move_size_nbs, q_p_move_size_nbc;
  std::vector<double> r_ms_sum, r_ms_n, q_p0_ms;
  size_t n_acpt_moves[7], n_moves[7];
  double acpt_goal;
  std::vector<size_t> move_inds_add, move_inds_rem, move_inds;
  std::vector<int64_t> move_inds_map;
  std::vector<unsigned char> move_isadd;
  unsigned char movesize;
  bool started;
  double k_move_size;
  double pves[3];
  std::vector<double> r_cm, r_om, xs;  /* RB scratch */
  Trace tr;
  /* delayed rejection (src/sampler.hpp:163-169, 272-281) */
  unsigned char delay_rejection = 0;
  ExhModel* exh = nullptr;
  std::vector<double> dr_model_probabilities, dr_q_add, dr_q_rem, dr_log_q_add_types;
  std::vector<unsigned char> dr_bit_to_normalized_order;

  Sampler(const bmg_options& opt, const Data* d, const PreXX* p, uint32_t seed_)
  : o(opt), data(d), pre(p), n_iter(0), do_n_iter(opt.do_n_iter), n_accepted(0),
    n_rao(opt.n_rao), n_rao_burnin(opt.n_rao_burnin), n_sample_tau2(opt.n_sample_tau2_and_missing),
    flat_proposal_dist(opt.flat_proposal_dist), adaptation(opt.adaptation),
    save_beta(opt.save_beta), thin(opt.thin), m_g(d->m_g), n_types(opt.n_types),
    use_types(opt.n_types > 1), seed(seed_), rng(seed_, d->n + opt.nu_sigma2),
    p_proposal_n(1), p_rao_n(0), dd_add(nullptr), dd_rem(nullptr), movesize(0),
    started(false), k_move_size(0)
  {
    std::vector<int> types(opt.types, opt.types + opt.n_types);
    dm = new DataModel(d, types);
    /* src/sampler.hpp:173-193 */
    double s2_sigma2 = (opt.s2_sigma2 > 0) ? opt.s2_sigma2
                       : d->var_y * (1 - opt.R2mode_sigma2) * (opt.nu_sigma2 + 2) / opt.nu_sigma2;
    double s2_tau2[4] = {0, 0, 0, 0};
    for (int t = 0; t < 4; ++t) {
      if (!dm->allow_terms(t)) continue;
      if (opt.s2_tau2[t] > 0) s2_tau2[t] = opt.s2_tau2[t];
      else
        s2_tau2[t] = opt.eh_tau2[t] * (opt.nu_tau2[t] - 2) /
                     (opt.nu_tau2[t] * (d->var_x + d->mean_x * d->mean_x) * (1 - opt.R2mode_sigma2));
    }
    std::vector<double> ite(d->m_e, opt.inv_tau2_e_val);
    ite[0] = opt.inv_tau2_e_const_val;
    prior = new Prior(d, dm, opt.types_prior, opt.e_qg, opt.var_qg, ite, opt.nu_sigma2, s2_sigma2,
                      opt.nu_tau2, s2_tau2, opt.mu_alpha, opt.use_individual_tau2);
    size_t cap = opt.max_model_size ? opt.max_model_size : 1024;
    cur = new Model(d, dm, prior, &stats, cap);
    nm = new Model(d, dm, prior, &stats, cap);
    exh = new ExhModel(d, dm, prior, &stats, cap);  /* src/sampler.hpp:203 */
    p_proposal.assign(m_g, 0.0);
    if (n_types > 1) p_proposal_types.assign(m_g * n_types, 0.0);
    p_rao.assign(m_g, 0.0);
    if (n_types > 1) p_rao_types.assign(m_g * n_types, 0.0);
    q_add.assign(m_g, 0.0);
    q_rem.assign(m_g, 0.0);
    p_r.assign(m_g, 0.0);
    if (use_types) {
      p_r_types.assign(m_g * n_types, 0.0);
      q_add_types.assign(m_g * n_types, 0.0);
      q_p_add_types.assign(m_g * n_types, 0.0);
    }
    q_add_min = 1.0 / (m_g - opt.e_qg);
    q_rem_min = 1.0 / opt.e_qg;
    max_move_size = (unsigned char)std::min(std::min(m_g, (size_t)255), (size_t)opt.max_move_size);
    delay_rejection = (unsigned char)std::min((size_t)max_move_size, (size_t)opt.delay_rejection);
    if (delay_rejection > 0) {
      dr_model_probabilities.assign((size_t)std::pow(2, delay_rejection), 0.0);
      dr_q_add.assign(delay_rejection, 0.0);
      dr_q_rem.assign(delay_rejection, 0.0);
      dr_log_q_add_types.assign(delay_rejection, 0.0);
      dr_bit_to_normalized_order.assign(delay_rejection, 0);
    }
    max_nbh = opt.max_SNP_neighborhood_size;
    p_move_size = opt.p_move_size;
    p_move_size_nbs = opt.p_move_size_nbs;
    p_move_size_nbc = opt.p_move_size_nbc;
    adapt_p_move_size = opt.adapt_p_move_size && max_move_size > 1;
    acpt_goal = opt.p_move_size_acpt_goal;
    move_inds_add.assign(max_move_size, 0);
    move_inds_rem.assign(max_move_size, 0);
    move_inds.assign(max_move_size, 0);
    move_inds_map.assign(max_move_size, 0);
    move_isadd.assign(max_move_size, 0);
    for (int i = 0; i < 7; ++i) { n_acpt_moves[i] = 0; n_moves[i] = 0; }
    n_acpt_moves[0] = n_acpt_moves[1] = n_acpt_moves[2] = 1;
    n_moves[0] = n_moves[1] = n_moves[2] = 2;
    q_p_move_size.assign(max_move_size, 0.0);
    r_ms_sum.assign(max_move_size, 0.0);
    r_ms_n.assign(max_move_size, 0.0);
    q_p0_ms.assign(max_move_size, 0.0);
    size_t mm2 = (max_move_size + 1) / 2;
    q_p_move_size_nbs.assign(mm2, 0.0);
    q_p_move_size_nbc.assign(max_move_size, 0.0);
    geometric_dist_cdf(max_move_size, p_move_size, q_p_move_size.data());
    geometric_dist_cdf((int)mm2, p_move_size_nbs, q_p_move_size_nbs.data());
    geometric_dist_cdf(max_move_size, p_move_size_nbc, q_p_move_size_nbc.data());
    r_cm.assign(d->n, 0.0);
    r_om.assign(d->n, 0.0);
    xs.assign(d->n, 1.0);
    initialize_p_proposal_flat();
  }
  ~Sampler()
  {
    delete dd_add; delete dd_rem; delete cur; delete nm; delete exh; delete prior; delete dm;
  }

  /* src/sampler.hpp:351-362 */
  void initialize_p_proposal_flat()
  {
    double val = prior->e_g() / (double)m_g;
    double vt = 1.0 / n_types;
    for (size_t i = 0; i < m_g; ++i) {
      p_proposal[i] = val;
      if (use_types)
        for (size_t t = 0; t < n_types; ++t) p_proposal_types[i * n_types + t] = vt;
    }
  }

  /* src/sampler.cpp:455-515 (PMV) */
  void compute_p_moves()
  {
    double pm[7] = {0.7, 0.15, 0.15, 0, 0, 0, 0};
    if (use_types) { pm[0] = 0.8; pm[1] = 0.1; pm[2] = 0.0; pm[3] = 0.1; }
    for (int i = 0; i < 7; ++i) p_moves[i] = pm[i];
    p_moves_cumsum[0] = p_moves[0];
    for (int i = 1; i < 7; ++i) p_moves_cumsum[i] = p_moves_cumsum[i - 1] + p_moves[i];
  }
  /* src/sampler.cpp:517-544 */
  void compute_proposal_dist()
  {
    for (size_t i = 0; i < m_g; ++i) q_add[i] = std::max(p_proposal[i], q_add_min);
  }
  void compute_proposal_types_dist()
  {
    for (size_t i = 0; i < m_g; ++i) {
      double val = std::max(p_proposal_types[i * n_types], q_add_min);
      q_add_types[i * n_types] = val;
      q_p_add_types[i * n_types] = val;
      for (size_t t = 1; t < n_types; ++t) {
        val = std::max(p_proposal_types[i * n_types + t], q_add_min);
        q_add_types[i * n_types + t] = val;
        q_p_add_types[i * n_types + t] = q_p_add_types[i * n_types + t - 1] + val;
      }
    }
  }

  /* src/sampler.cpp:32-261 */
  double* logodds_out = nullptr;  // when set: the log posterior odds of inclusion per SNP

  void p_raoblackwell(const std::vector<double>& y_hat, double* pr, double* prt)
  {
    const Model* cm = cur;
    const double s2x2 = 2 * cm->sigma2;
    const size_t nt = dm->n_types;
    const bool ut = (nt > 1);
    const size_t n = dm->n;
    for (size_t i = 0; i < n; ++i) r_cm[i] = data->y[i] - y_hat[i];
    double s = 0;
    for (size_t i = 0; i < n; ++i) s += r_cm[i];
    double mr_cm = s / n;
    int Ns[5];
    std::memcpy(Ns, cm->Ns, sizeof(Ns));
    size_t n_loci = cm->size();
    double lmp_add[5] = {0, 0, 0, 0, 0}, lmp_rem[5][5];
    for (int t = 0; t < 5; ++t) {
      if (!dm->allow_types(t)) continue;
      if ((size_t)(Ns[t] + 1) <= m_g) lmp_add[t] = prior->compute_log_change_on_add(Ns, (int)n_loci, t);
      Ns[t]--;
      n_loci--;
      if (Ns[t] >= 0)
        for (int j = 0; j < 5; ++j)
          if (dm->allow_types(j)) lmp_rem[t][j] = prior->compute_log_change_on_add(Ns, (int)n_loci, j);
      Ns[t]++;
      n_loci++;
    }
    double itv[4] = {0, 0, 0, 0};
    if (!prior->use_individual_tau2)
      for (int t = 0; t < 4; ++t)
        if (dm->allow_terms(t)) itv[t] = prior->inv_tau2_alpha2[t];
    std::vector<double> pxx(pre->offset);
    for (size_t i = 0; i < m_g; ++i) {
      const std::vector<double>* res;
      double mr, det, et, slq;
      const double* lmp;
      int32_t mi = cm->model_inds[i];
      if (prior->use_individual_tau2)
        for (int t = 0; t < 4; ++t)
          if (dm->allow_terms(t)) itv[t] = prior->sample_single_inv_tau2_from_prior_times_alpha2(t, rng);
      if (mi < 0) {
        res = &r_cm;
        mr = mr_cm;
        lmp = lmp_add;
      } else {
        unsigned int xi = cm->x_ind1[mi];
        int type = dm->types[cm->type_inds[mi]];
        if (prior->use_individual_tau2) {
          if (type == AH) {
            itv[A] = cm->inv[xi];
            itv[H] = cm->inv[cm->x_ind2[mi]];
          } else {
            itv[type] = cm->inv[xi];
          }
        }
        r_om = r_cm;
        double b = cm->beta[xi];
        for (size_t k = 0; k < n; ++k) r_om[k] += b * cm->x[xi * n + k];
        if (type == AH) {
          xi = cm->x_ind2[mi];
          b = cm->beta[xi];
          for (size_t k = 0; k < n; ++k) r_om[k] += b * cm->x[xi * n + k];
        }
        res = &r_om;
        double so = 0;
        for (size_t k = 0; k < n; ++k) so += r_om[k];
        mr = so / n;
        lmp = lmp_rem[type];
      }
      double max_types = -INFINITY;
      std::memcpy(pxx.data(), &pre->xx[i * pre->offset], pre->offset * sizeof(double));
      dm->update_prexx_cov(i, pxx.data());
      for (size_t t = 0; t < nt; ++t) {
        int type = dm->types[t];
        if (type == AH) {
          double sa = pxx[0], va = pxx[1] + itv[A], sh = pxx[2], vh = pxx[3] + itv[H];
          double vah = pxx[pre->offset - 1];
          slq = -log(itv[A]) - log(itv[H]);
          dm->get_genotypes(A, i, xs.data());
          double rxa = ddot(n, xs.data(), res->data()) - sa * mr;
          dm->get_genotypes(H, i, xs.data());
          double rxh = ddot(n, xs.data(), res->data()) - sh * mr;
          det = va * vh - vah * vah;
          et = rxa * rxa * vh - 2.0 * rxa * rxh * vah + rxh * rxh * va;
          et /= det;
        } else {
          size_t off = pre->offset_type[type];
          double sv = pxx[off];
          det = pxx[off + 1] + itv[type];
          slq = -log(itv[type]);
          dm->get_genotypes(type, i, xs.data());
          double rx = ddot(n, xs.data(), res->data()) - sv * mr;
          et = (rx * rx) / det;
        }
        double p = et / s2x2 - 0.5 * (log(det) + slq) + lmp[type];
        if (ut) {
          if (p > max_types) max_types = p;
          prt[i * nt + t] = p;
        } else {
          if (logodds_out) logodds_out[i] = p;
          p = exp(p);
          pr[i] = std::isfinite(p) ? p / (1 + p) : 1;
        }
      }
      if (ut) {
        if (!std::isfinite(max_types)) {
          if (std::isnan(max_types)) throw std::runtime_error("raob max_types is nan");
          if (max_types > 0) {
            double st = 0;
            for (size_t t = 0; t < nt; ++t) {
              double& q = prt[i * nt + t];
              q = (!std::isfinite(q) && q > 0) ? 1 : 0;
              st += q;
            }
            for (size_t t = 0; t < nt; ++t) prt[i * nt + t] /= st;
            pr[i] = 1;
          } else {
            for (size_t t = 0; t < nt; ++t) prt[i * nt + t] = 1.0 / nt;
            pr[i] = 0;
          }
          if (logodds_out) logodds_out[i] = max_types;
          continue;
        }
        double st = 0;
        for (size_t t = 0; t < nt; ++t) {
          prt[i * nt + t] = exp(prt[i * nt + t] - max_types);
          st += prt[i * nt + t];
        }
        for (size_t t = 0; t < nt; ++t) prt[i * nt + t] /= st;
        if (logodds_out) logodds_out[i] = log(st) + max_types;
        st = exp(log(st) + max_types);
        pr[i] = std::isfinite(st) ? st / (1 + st) : 1;
      }
    }
  }

  /* The exact change of the current model's log marginal likelihood from
     adding single term t of SNP j, for every SNP outside the model and every
     allowed single term (A, H, D, R in that order): the formulas of
     Model::update_likelihood_on_add (src/model.hpp:432-506) evaluated on the
     new column alone, with the chain's shared prior precision of the term;
     the model is left unchanged.  NaN for SNPs in the model. */
  void schur_scan(double* out, double* itv_out)
  {
    const Model* m = cur;
    const size_t n = dm->n, k = m->xcols;
    std::vector<int> terms;
    for (int t = 0; t < 4; ++t)
      if (dm->allow_terms(t)) terms.push_back(t);
    std::vector<double> xcol(n), g(k > 0 ? k : 1);
    for (int t = 0; t < 4; ++t) itv_out[t] = dm->allow_terms(t) ? prior->inv_tau2_alpha2[t] : NAN;
    for (size_t j = 0; j < m_g; ++j) {
      for (size_t u = 0; u < terms.size(); ++u) {
        double& o = out[j * terms.size() + u];
        if (m->model_inds[j] >= 0) {
          o = NAN;
          continue;
        }
        const int t = terms[u];
        const double inv_val = prior->inv_tau2_alpha2[t];
        dm->get_genotypes(t, j, xcol.data());
        const double xy = ddot(n, xcol.data(), data->y.data());
        const double xxc = ddot(n, xcol.data(), xcol.data());
        cblas_dgemv(CblasColMajor, CblasTrans, (int)n, (int)k, 1.0, m->x.data(), (int)n, xcol.data(), 1, 0.0,
                    g.data(), 1);
        cblas_dtrsv(CblasColMajor, CblasUpper, CblasTrans, CblasNonUnit, (int)k, m->l.data(), (int)m->cap,
                    g.data(), 1);
        const double lmm2 = xxc + inv_val - ddot(k, g.data(), g.data());
        if (lmm2 <= 0) {
          o = -INFINITY;
          continue;
        }
        const double lcc = sqrt(lmm2);
        const double vc = (xy - ddot(k, g.data(), m->v.data())) / lcc;
        const double syx2 = m->syx_plus_vs2 - vc * vc;
        o = 0.5 * log(inv_val) - log(lcc) + prior->minus_n_plus_nu_2 * (log(syx2) - log(m->syx_plus_vs2));
      }
    }
  }

  /* src/sampler.cpp:264-453 */
  void sample_missing()
  {
    const size_t n = dm->n;
    const double s2x2 = cur->sigma2 * 2;
    double lprior[3], lik[3];
    std::vector<double> yh(n, 0.0), res(n);
    cblas_dgemv(CblasColMajor, CblasNoTrans, (int)n, (int)cur->xcols, 1.0, cur->x.data(), (int)n,
                cur->beta.data(), 1, 0.0, yh.data(), 1);
    for (size_t i = 0; i < n; ++i) res[i] = data->y[i] - yh[i];
    double r2 = 0;
    for (size_t i = 0; i < n; ++i) r2 += res[i] * res[i];
    const std::vector<double>& b = cur->beta;
    for (size_t i = 0; i < cur->size(); ++i) {
      uint32_t ind = cur->loci[i];
      if (data->miss_loc[ind].empty()) continue;
      int type = dm->types[cur->type_inds[i]];
      unsigned x1 = cur->x_ind1[i];
      unsigned x2 = (type == AH) ? cur->x_ind2[i] : 0;
      double* t1 = &cur->x[x1 * n];
      double* t2 = &cur->x[x2 * n];
      const std::vector<double>& mp = data->miss_prior[ind];
      lprior[0] = log(mp[0]);
      lprior[1] = log(mp[1] - mp[0]);
      lprior[2] = log(mp[2] - mp[1]);
      const std::vector<size_t>& ml = data->miss_loc[ind];
      for (size_t j = 0; j < ml.size(); ++j) {
        size_t im = ml[j];
        double old2 = res[im] * res[im];
        double nt;
        for (int k = 0; k < 3; ++k) {
          double gk;
          switch (type) {
            case A: case AH: gk = (double)k; break;
            case H: gk = (double)(k == 1); break;
            case R: gk = (double)(k == 2); break;
            default: gk = (double)(k > 0); break;
          }
          nt = res[im] - b[x1] * (gk - t1[im]);
          if (type == AH) nt -= b[x2] * ((double)(k == 1) - t2[im]);
          lik[k] = lprior[k] - (r2 + nt * nt - old2) / s2x2;
        }
        lik[1] -= lik[0];
        lik[2] -= lik[0];
        lik[0] = 1;
        lik[1] = exp(lik[1]) + lik[0];
        lik[2] = exp(lik[2]) + lik[1];
        int k = sample_discrete_naive(lik, 3, rng);
        dm->miss_val[ind][j] = (char)k;
        switch (type) {
          case A: break;
          case H: k = (k == 1); break;
          case R: k = (k == 2); break;
          case D: k = (k > 0); break;
          default: break;
        }
        yh[im] += b[x1] * ((double)k - t1[im]);
        t1[im] = (double)k;
        if (type == AH) {
          k = (k == 1);
          yh[im] += b[x2] * ((double)k - t2[im]);
          t2[im] = (double)k;
        }
        res[im] = data->y[im] - yh[im];
        r2 += res[im] * res[im] - old2;
      }
    }
    for (size_t i = 0; i < cur->size(); ++i) {
      uint32_t ind = cur->loci[i];
      int type = dm->types[cur->type_inds[i]];
      if (data->miss_loc[ind].empty()) continue;
      for (int pass = 0; pass < (type == AH ? 2 : 1); ++pass) {
        unsigned xi = pass ? cur->x_ind2[i] : cur->x_ind1[i];
        const double* xnew = &cur->x[xi * n];
        const double* xold = &nm->x[xi * n];
        const std::vector<size_t>& ml = data->miss_loc[ind];
        for (size_t j = 0; j < ml.size(); ++j) {
          size_t im = ml[j];
          cur->xy[xi] += data->y[im] * (xnew[im] - xold[im]);
          unsigned k = 0;
          for (; k < xi; ++k)
            if (k < dm->m_e || !dm->genotype_missing(im, cur->x_ind_to_g_ind[k]))
              cur->XX(k, xi) += xnew[im] * cur->x[k * n + im] - xold[im] * nm->x[k * n + im];
          for (; k < cur->xcols; ++k)
            cur->XX(xi, k) += xnew[im] * cur->x[k * n + im] - xold[im] * nm->x[k * n + im];
        }
      }
    }
    cur->mu_beta_computed = false;
  }

  /* src/sampler.hpp:500-515 */
  void prepare_add_new_term_nm(int type, double* itv)
  {
    if (type == AH) {
      itv[0] = prior->sample_single_inv_tau2_from_prior_times_alpha2(A, rng);
      itv[1] = prior->sample_single_inv_tau2_from_prior_times_alpha2(H, rng);
    } else {
      itv[0] = prior->sample_single_inv_tau2_from_prior_times_alpha2(type, rng);
    }
  }
  void prepare_add_new_term(size_t ind, int type, double* itv)
  {
    dm->sample_missing_single((uint32_t)ind, rng);
    prepare_add_new_term_nm(type, itv);
  }

  /* src/sampler.hpp:899-1123 */
  unsigned char do_multistep_additions_and_removals()
  {
    movesize = (unsigned char)(sample_discrete_naive(q_p_move_size.data(), max_move_size, rng) + 1);
    double lqf = 0.0, lqb = 0.0, lmpc = 0.0;
    unsigned char ms_rem = 0;
    prepare_addrem(lqf, ms_rem, movesize);
    do_addrem(lqf, lqb, lmpc, movesize);
    backward_prepare_addrem(lqb, movesize);
    double log_r = lqb - lqf;
    log_r += lmpc + nm->log_likelihood_ - cur->log_likelihood_;
    if (delay_rejection == 0) r_ms_sum[movesize - 1] += (log_r >= 0 ? 1.0 : exp(log_r));
    r_ms_n[movesize - 1] += 1.0;
    if (log_r >= 0 || log(rng.rand_01()) <= log_r) {
      cur->copy_from(*nm);
      if (delay_rejection != 0) r_ms_sum[movesize - 1] += 1.0;
      return movesize;
    }
    /* the delayed rejection can propose the current model only for moves of
       more than one SNP */
    if (movesize <= delay_rejection && movesize > 1) return delayed_rejection(ms_rem);
    nm->copy_from(*cur);
    for (unsigned char i = 0; i < movesize; ++i) {
      size_t ind = move_inds[i];
      if (move_isadd[i]) { dd_add->remdate(ind); dd_rem->adddate(ind); }
      else { dd_add->adddate(ind); dd_rem->remdate(ind); }
    }
    return 0;
  }
  /* src/sampler.hpp:1009-1028 (also :1571-1595): each sub-model i below
     2^(movesize-1) is paired with its complement; the pair's weight is the
     difference of their probabilities, carried by the likelier one (the
     other's entry records which: -1 when the complement, 1 when i).  Samples
     a pair by its cumulative weight and returns the sub-model that carries
     it. */
  unsigned long dr_sample_pair(double max_log_model)
  {
    unsigned long nmodels = (unsigned long)std::pow(2, movesize);
    unsigned long mask = nmodels - 1;
    double* pm = dr_model_probabilities.data();
    double sum = 0.0;
    for (unsigned long i = 0; i < nmodels / 2; ++i) {
      unsigned int j = (~i) & mask;
      double a = pm[j] - pm[i];
      if (a > 0) {
        pm[i] = exp(pm[j] - max_log_model) * (1 - exp(-a));
        pm[j] = -1.0;
      } else {
        pm[i] = exp(pm[i] - max_log_model) * (1 - exp(a));
        pm[j] = 1.0;
      }
      pm[i] += sum;
      sum = pm[i];
    }
    unsigned long sampled_model = sample_discrete(pm, nmodels / 2, (int)movesize / 2 - 3, rng);
    if (pm[(~sampled_model) & mask] < 0) sampled_model = (~sampled_model) & mask;
    return sampled_model;
  }

  /* src/sampler.hpp:1547-1618: the same second stage after a rejected
     state change of movesize > 1 SNPs near a central in-model SNP; sub-model
     bits are the added SNPs then the removed ones, and each sub-model's
     probability includes choosing the central SNP among its in-model SNPs */
  unsigned char delayed_rejection_statechange(unsigned char ms_add, unsigned char ms_rem)
  {
    size_t const_loci = cur->size() - ms_rem;
    unsigned long newmodel_binary = ((1 << ms_add) - 1);
    for (unsigned char i_move = 0; i_move < ms_rem; ++i_move) {
      size_t ind = move_inds_rem[i_move];
      int cmi = cur->model_inds[ind];
      int t_ind = cur->type_inds[cmi];
      if (dm->types[t_ind] == AH) {
        double itv2[2] = {cur->inv[cur->x_ind1[cmi]], cur->inv[cur->x_ind2[cmi]]};
        nm->add_term((uint32_t)ind, t_ind, itv2);
      } else {
        double itv1 = cur->inv[cur->x_ind1[cmi]];
        nm->add_term((uint32_t)ind, t_ind, &itv1);
      }
    }
    exh->update_to_model(*nm, const_loci);
    double max_log_model;
    compute_exhaustive_modelset(movesize, exh, dr_model_probabilities.data(), max_log_model);
    unsigned long nmodels = (unsigned long)std::pow(2, movesize);
    unsigned long mask = nmodels - 1;
    for (unsigned int i = 0; i < nmodels; ++i)
      dr_model_probabilities[i] -= log(const_loci + __builtin_popcount(i));
    unsigned long sampled_model = dr_sample_pair(max_log_model);
    unsigned char moved = 0;
    if (sampled_model == ((~newmodel_binary) & mask)) {
      nm->copy_from(*cur);
    } else {
      for (unsigned char i_move = 0; i_move < movesize; ++i_move) {
        if (1 == ((sampled_model >> i_move) & 1)) {
          if (1 == ((newmodel_binary >> i_move) & 1)) {
            ++moved;
            size_t ind = move_inds_add[i_move];
            dd_add->adddate(ind);
            dd_rem->remdate(ind);
          }
        } else {
          if (0 == ((newmodel_binary >> i_move) & 1)) {
            ++moved;
            size_t ind = move_inds_rem[i_move - ms_add];
            dd_add->remdate(ind);
            dd_rem->adddate(ind);
          }
        }
      }
      unsigned long removals = mask & sampled_model;
      for (unsigned char i = 0; i < movesize; ++i) {
        if ((removals & 1) == 0) {
          nm->remove_term((int)(const_loci + i));
          --const_loci;
        }
        removals >>= 1;
      }
      cur->copy_from(*nm);
    }
    return moved;
  }

  /* src/sampler.hpp:929-1098: after a rejected move of movesize > 1 SNPs,
     sample among all 2^movesize sub-models of the involved SNPs (the current
     and the proposed model excepted), pairing each sub-model with its
     complement so the second stage keeps detailed balance */
  unsigned char delayed_rejection(unsigned char ms_rem)
  {
    size_t const_loci = cur->size() - ms_rem;
    unsigned char ms_add = movesize - ms_rem;
    double z_add = dd_add->total_w;
    double z_rem = dd_rem->total_w;
    unsigned long newmodel_binary = ((1 << ms_add) - 1);
    for (unsigned char i_move = 0; i_move < movesize; ++i_move) {
      size_t ind = move_inds[i_move];
      if (move_isadd[i_move]) {
        z_add += q_add[ind];
        z_rem -= q_rem[ind];
      } else {
        int cmi = cur->model_inds[ind];
        int t_ind = cur->type_inds[cmi];
        if (dm->types[t_ind] == AH) {
          double itv2[2] = {cur->inv[cur->x_ind1[cmi]], cur->inv[cur->x_ind2[cmi]]};
          nm->add_term((uint32_t)ind, t_ind, itv2);
        } else {
          double itv1 = cur->inv[cur->x_ind1[cmi]];
          nm->add_term((uint32_t)ind, t_ind, &itv1);
        }
      }
    }
    for (unsigned char i_move = 0; i_move < movesize; ++i_move) {
      size_t ind = (size_t)move_inds_map[i_move];
      size_t model_ind = (size_t)nm->model_inds[ind];
      dr_bit_to_normalized_order[model_ind - const_loci] = i_move;
      dr_q_add[i_move] = q_add[ind];
      dr_q_rem[i_move] = q_rem[ind];
      if (n_types > 1) {
        unsigned char t_ind = nm->type_inds[nm->model_inds[ind]];
        dr_log_q_add_types[i_move] = log(q_add_types[ind * n_types + t_ind] / q_p_add_types[ind * n_types + n_types - 1]);
      }
    }
    exh->update_to_model(*nm, const_loci);
    double max_log_model;
    compute_exhaustive_modelset(movesize, exh, dr_model_probabilities.data(), max_log_model);
    compute_proposal_probs_for_exh_modelset(use_types, movesize, dr_bit_to_normalized_order.data(), dr_q_add.data(),
                                            dr_q_rem.data(), z_add, z_rem, const_loci, m_g,
                                            dr_log_q_add_types.data(), dr_model_probabilities.data());
    unsigned long nmodels = (unsigned long)std::pow(2, movesize);
    unsigned long mask = nmodels - 1;
    unsigned long sampled_model = dr_sample_pair(max_log_model);
    unsigned char moved = 0;
    if (sampled_model == ((~newmodel_binary) & mask)) {
      nm->copy_from(*cur);
      for (unsigned char i_move = 0; i_move < movesize; ++i_move) {
        size_t ind = move_inds[i_move];
        if (move_isadd[i_move]) { dd_add->remdate(ind); dd_rem->adddate(ind); }
        else { dd_add->adddate(ind); dd_rem->remdate(ind); }
      }
    } else {
      for (unsigned char i_move = 0; i_move < movesize; ++i_move) {
        if (1 == ((sampled_model >> i_move) & 1)) {
          if (0 == ((newmodel_binary >> i_move) & 1)) {
            size_t ind = (size_t)move_inds_map[dr_bit_to_normalized_order[i_move]];
            dd_add->adddate(ind);
            dd_rem->remdate(ind);
          } else {
            ++moved;
          }
        } else {
          if (1 == ((newmodel_binary >> i_move) & 1)) {
            size_t ind = (size_t)move_inds_map[dr_bit_to_normalized_order[i_move]];
            dd_add->remdate(ind);
            dd_rem->adddate(ind);
          } else {
            ++moved;
          }
        }
      }
      unsigned long removals = mask & sampled_model;
      for (unsigned char i = 0; i < movesize; ++i) {
        if ((removals & 1) == 0) {
          nm->remove_term((int)(const_loci + i));
          --const_loci;
        }
        removals >>= 1;
      }
      r_ms_sum[movesize - 1] += (double)moved / (double)movesize;
      cur->copy_from(*nm);
    }
    return moved;
  }

  /* src/sampler.hpp:1126-1165 */
  void prepare_addrem(double& lqf, unsigned char& n_rem, unsigned char ms)
  {
    size_t max_adds = m_g - cur->size(), max_rems = cur->size();
    n_rem = 0;
    for (unsigned char i = 0; i < ms; ++i) {
      bool add;
      if (max_rems == 0) add = true;
      else if (max_adds == 0) add = false;
      else { lqf += kLogHalf; add = (rng.rand_01() < 0.5); }
      if (add) {
        --max_adds;
        move_isadd[i] = 1;
        size_t ind = dd_add->sample();
        move_inds[i] = ind;
        move_inds_map[i] = (int64_t)ind;
        lqf += log(q_add[ind]) - log(dd_add->total_w);
        dd_add->adddate(ind);
      } else {
        ++n_rem;
        --max_rems;
        move_isadd[i] = 0;
        size_t ind = dd_rem->sample();
        move_inds[i] = ind;
        move_inds_map[i] = -1;
        lqf += log(q_rem[ind]) - log(dd_rem->total_w);
        dd_rem->adddate(ind);
      }
    }
  }
  /* src/sampler.hpp:1168-1202 */
  void backward_prepare_addrem(double& lqb, unsigned char ms)
  {
    size_t max_adds = m_g - nm->size(), max_rems = nm->size();
    double w_add = dd_add->total_w, w_rem = dd_rem->total_w;
    int last_rem_pos = ms - 1;
    for (unsigned char i = 0; i < ms; ++i) {
      if (max_adds > 0 && max_rems > 0) lqb += kLogHalf;
      size_t ind;
      if (move_isadd[i]) {
        --max_rems;
        while (!move_isadd[last_rem_pos]) --last_rem_pos;
        ind = (size_t)move_inds_map[last_rem_pos];
        --last_rem_pos;
        lqb += log(q_rem[ind]) - log(w_rem);
        w_rem -= q_rem[ind];
      } else {
        --max_adds;
        ind = (size_t)move_inds_map[i];
        lqb += log(q_add[ind]) - log(w_add);
        w_add -= q_add[ind];
      }
    }
  }
  /* src/sampler.hpp:1204-1268 */
  void do_addrem(double& lqf, double& lqb, double& lmpc, unsigned char ms)
  {
    int last_map_pos = ms - 1;
    for (unsigned char i = 0; i < ms; ++i) {
      if (move_isadd[i]) continue;
      size_t ind = move_inds[i];
      dd_add->remdate(ind);
      while (move_inds_map[last_map_pos] >= 0) --last_map_pos;
      move_inds_map[last_map_pos] = (int64_t)ind;
      int mi = nm->model_inds[ind];
      int t_ind = nm->type_inds[mi];
      int type = dm->types[t_ind];
      lmpc += prior->compute_log_change_on_rem(nm->Ns, (int)nm->size(), type);
      if (use_types) lqb += log(q_add_types[ind * n_types + t_ind] / q_p_add_types[ind * n_types + n_types - 1]);
      nm->remove_term(mi);
    }
    double itv[2];
    for (unsigned char i = 0; i < ms; ++i) {
      if (!move_isadd[i]) continue;
      size_t ind = move_inds[i];
      dd_rem->remdate(ind);
      int t_ind = 0;
      if (use_types) t_ind = sample_discrete_naive(&q_p_add_types[ind * n_types], (int)n_types, rng);
      int type = dm->types[t_ind];
      lmpc += prior->compute_log_change_on_add(nm->Ns, (int)nm->size(), type);
      if (use_types) lqf += log(q_add_types[ind * n_types + t_ind] / q_p_add_types[ind * n_types + n_types - 1]);
      prepare_add_new_term(ind, type, itv);
      nm->add_term((uint32_t)ind, t_ind, itv);
    }
  }

  /* src/sampler.hpp:1271-1418 */
  unsigned char do_switch_of_nearby_snps()
  {
    size_t full = m_g - cur->size();
    size_t mm2 = (max_move_size + 1) / 2;
    unsigned char mms = (unsigned char)std::min(mm2, (full + 1) / 2);
    mms = (unsigned char)std::min((size_t)mms, cur->size());
    movesize = (unsigned char)(sample_discrete_naive(q_p_move_size_nbs.data(), mms, rng) + 1);
    size_t nbh = std::max((size_t)1, (full - movesize) / 2);
    nbh = std::min(max_nbh, nbh);
    for (unsigned char im = 0; im < movesize; ++im) {
      size_t mir = (size_t)std::floor(rng.rand_01() * nm->size());
      size_t ind_rem = nm->loci[mir];
      move_inds_rem[im] = ind_rem;
      size_t ind_add;
      int j = 0;
      int mv = (int)std::floor(rng.rand_01() * nbh) + 1;
      if (rng.rand_01() < 0.5) {
        ind_add = ind_rem;
        j = 0;
        while (j < mv) {
          ++ind_add;
          if (ind_add < m_g) {
            if (cur->model_inds[ind_add] < 0) ++j;
          } else {
            break;
          }
        }
        if (ind_add == m_g) {
          ind_add = ind_rem;
          mv = mv + mv - j;
          j = 0;
          while (j < mv) {
            --ind_add;
            while (cur->model_inds[ind_add] >= 0) --ind_add;
            ++j;
          }
        }
      } else {
        ind_add = ind_rem;
        j = 0;
        if (ind_add > 0) {
          while (j < mv) {
            --ind_add;
            if (ind_add > 0) {
              if (cur->model_inds[ind_add] < 0) ++j;
            } else {
              break;
            }
          }
        }
        if (j < mv) {
          if (cur->model_inds[ind_add] < 0) ++j;
          if (j < mv) {
            ind_add = ind_rem;
            mv = mv + mv - j;
            j = 0;
            while (j < mv) {
              ++ind_add;
              while (cur->model_inds[ind_add] >= 0) ++ind_add;
              ++j;
            }
          }
        }
      }
      move_inds_add[im] = ind_add;
      int t_ind = nm->type_inds[mir];
      nm->remove_term((int)mir);
      cur->model_inds[ind_add] = t_ind;  /* the reference's temporary marking */
    }
    double itv[2];
    for (unsigned char im = 0; im < movesize; ++im) {
      size_t ind_add = move_inds_add[im];
      int t_ind = (char)cur->model_inds[ind_add];
      int type = dm->types[t_ind];
      prepare_add_new_term(ind_add, type, itv);
      nm->add_term((uint32_t)ind_add, t_ind, itv);
      cur->model_inds[ind_add] = -1;
    }
    double log_r = nm->log_likelihood_ - cur->log_likelihood_;
    if (log_r >= 0 || log(rng.rand_01()) <= log_r) {
      cur->copy_from(*nm);
      for (unsigned char im = 0; im < movesize; ++im) {
        dd_add->remdate(move_inds_rem[im]);
        dd_rem->adddate(move_inds_rem[im]);
        dd_add->adddate(move_inds_add[im]);
        dd_rem->remdate(move_inds_add[im]);
      }
      return 2 * movesize;
    }
    nm->copy_from(*cur);
    return 0;
  }

  /* src/sampler.hpp:1421-1669 (delayed rejection off) */
  unsigned char do_statechange_of_nearby_snps()
  {
    size_t mms = std::min(max_nbh * 2, std::min(m_g - 1, (size_t)max_move_size));
    movesize = (unsigned char)(sample_discrete_naive(q_p_move_size_nbc.data(), (int)mms, rng) + 1);
    // src/sampler.hpp:1441 takes min(max_nbh, m_g / 2), which wraps below
    // index 0 (UB) when 2 nbh + 1 > m_g; capped at (m_g - 1) / 2 as on the GPU
    size_t nbh = std::min(max_nbh, (m_g - 1) / 2);
    size_t mic = (size_t)std::floor(rng.rand_01() * nm->size());
    size_t ind_c = nm->loci[mic];
    std::vector<size_t> perm(2 * nbh);
    for (size_t i = 0; i < 2 * nbh; ++i) perm[i] = i;
    size_t wrap = ind_c + nbh;
    if (ind_c < nbh) wrap += (nbh - ind_c);
    else if (wrap > m_g - 1) wrap = m_g - 1;
    for (unsigned char im = 0; im < movesize; ++im) {
      size_t ind = (size_t)std::floor(rng.rand_01() * (nbh * 2 - im)) + im;
      std::swap(perm[im], perm[ind]);
    }
    unsigned char ms_rem = 0, ms_add = 0;
    for (unsigned char im = 0; im < movesize; ++im) {
      size_t ind = perm[im] + ind_c + 1;
      if (ind > wrap) ind = ind_c - (ind - wrap);
      if (nm->model_inds[ind] < 0) move_inds_add[ms_add++] = ind;
      else move_inds_rem[ms_rem++] = ind;
    }
    double lmpc = 0.0;
    for (unsigned char im = 0; im < ms_rem; ++im) {
      int mir = nm->model_inds[move_inds_rem[im]];
      int type = dm->types[nm->type_inds[mir]];
      lmpc += prior->compute_log_change_on_rem(nm->Ns, (int)nm->size(), type);
      nm->remove_term(mir);
    }
    double itv[2];
    int t_ind = nm->type_inds[mic];
    int type = dm->types[t_ind];
    for (unsigned char im = 0; im < ms_add; ++im) {
      size_t ind_add = move_inds_add[im];
      lmpc += prior->compute_log_change_on_add(nm->Ns, (int)nm->size(), type);
      prepare_add_new_term(ind_add, type, itv);
      nm->add_term((uint32_t)ind_add, t_ind, itv);
    }
    double log_r = lmpc + nm->log_likelihood_ - cur->log_likelihood_;
    log_r += log((double)cur->size()) - log((double)nm->size());
    if (log_r >= 0 || log(rng.rand_01()) <= log_r) {
      cur->copy_from(*nm);
      for (unsigned char im = 0; im < ms_add; ++im) {
        dd_add->adddate(move_inds_add[im]);
        dd_rem->remdate(move_inds_add[im]);
      }
      for (unsigned char im = 0; im < ms_rem; ++im) {
        dd_add->remdate(move_inds_rem[im]);
        dd_rem->adddate(move_inds_rem[im]);
      }
      return movesize;
    }
    if (movesize <= delay_rejection && movesize > 1) return delayed_rejection_statechange(ms_add, ms_rem);
    nm->copy_from(*cur);
    return 0;
  }

  /* src/sampler.hpp:1672-1713 */
  unsigned char do_switch_of_types()
  {
    movesize = 1;
    int mi = (int)round((cur->size() - 1) * rng.rand_01());
    size_t ind = cur->loci[mi];
    size_t tr = cur->type_inds[mi];
    const double* qa = &q_add_types[ind * n_types];
    q_p_add_types_tmp[0] = (tr == 0) ? 0 : qa[0];
    for (size_t i = 1; i < n_types; ++i)
      q_p_add_types_tmp[i] = q_p_add_types_tmp[i - 1] + ((tr == i) ? 0 : qa[i]);
    int ta = sample_discrete_naive(q_p_add_types_tmp, (int)n_types, rng);
    int type_add = dm->types[ta], type_rem = dm->types[tr];
    double itv[2];
    nm->remove_term(mi);
    prepare_add_new_term_nm(type_add, itv);
    nm->add_term((uint32_t)ind, ta, itv);
    double r = prior->compute_log_change_on_swi(cur->Ns, type_add, type_rem) +
               nm->log_likelihood_ - cur->log_likelihood_ -
               log(qa[ta] / q_p_add_types_tmp[n_types - 1]) +
               log(qa[tr] / (q_p_add_types[ind * n_types + n_types - 1] - qa[ta]));
    if (r >= 0 || log(rng.rand_01()) <= r) {
      cur->copy_from(*nm);
      return 1;
    }
    nm->copy_from(*cur);
    return 0;
  }

  /* src/sampler.hpp:1715-1769 */
  void adapt_p_move_size_acptrate(double t)
  {
    double ar = (double)n_acpt_moves[0] / (double)n_moves[0];
    p_move_size = p_move_size + (acpt_goal - ar) / t;
    p_move_size = std::max(std::min(p_move_size, 0.99), 0.01);
    n_acpt_moves[0] = 1;
    n_moves[0] = 2;
  }
  void adapt_p_move_size_jd_mb()
  {
    unsigned char mx = max_move_size;
    double q = 1 - p_move_size;
    double zp = 1 - std::pow(q, mx);
    double q_p = p_move_size / zp;
    for (unsigned i = 0; i < mx; ++i) { q_p0_ms[i] += q_p; q_p *= q; }
    double p_best = 0.01, p = 0.01, h_best = -INFINITY, h;
    double step = 0.98 / 49.0, ratio;
    for (int j = 0; j < 50; ++j) {
      h = 0.0; zp = 0.0; q = 1.0 - p; q_p = p;
      for (unsigned i = 0; i < mx; ++i) {
        ratio = q_p / q_p0_ms[i];
        h += (i + 1) * r_ms_sum[i] * ratio;
        zp += r_ms_n[i] * ratio;
        q_p *= q;
      }
      h /= zp;
      if (h > h_best) { h_best = h; p_best = p; }
      p += step;
    }
    p_move_size = p_best;
  }

  /* src/sampler.cpp:551-620: everything sample() does before its loop */
  void start()
  {
    if (!std::isfinite(cur->log_likelihood_))
      throw std::runtime_error("Sampler cannot start from non-finite likelihood.");
    pves[0] = pves[1] = pves[2] = 0.0;
    k_move_size = 1000.0 / n_rao_burnin;
    nm->copy_from(*cur);
    compute_proposal_dist();
    for (size_t i = 0; i < m_g; ++i) q_rem[i] = std::max(1 - p_proposal[i], q_rem_min);
    dd_add = new DD(q_add.data(), m_g, &rng);
    dd_rem = new DD(q_rem.data(), m_g, &rng);
    for (size_t i = 0; i < m_g; ++i) dd_rem->adddate(i);
    if (use_types) compute_proposal_types_dist();
    compute_p_moves();
    cur->sample_beta_sigma2(rng);
    sample_missing();
    prior->sample_alpha_and_tau2(cur, rng);
    cur->compute_log_likelihood();
    nm->copy_from(*cur);
    started = true;
  }

  /* src/sampler.cpp:626-834: one iteration */
  void iterate(size_t iter)
  {
    if ((iter + 1) % n_sample_tau2 == 0) {
      sample_missing();
      prior->sample_alpha_and_tau2(cur, rng);
      cur->compute_log_likelihood();
      nm->copy_from(*cur);
    }
    unsigned char move = (unsigned char)sample_discrete_naive(p_moves_cumsum, 7, rng);
    unsigned char jd = 0;
    switch (move) {
      case 0: jd = do_multistep_additions_and_removals(); break;
      case 1:
        if (cur->size() > 0 && cur->size() < (m_g - 1)) jd = do_switch_of_nearby_snps();
        break;
      case 2:
        if (cur->size() > 0 && m_g > 2) jd = do_statechange_of_nearby_snps();
        break;
      case 3:
        if (cur->size() > 0) jd = do_switch_of_types();
        break;
      default: throw std::logic_error("move not supported on this path");
    }
    ++n_moves[move];
    n_acpt_moves[move] += jd > 0;
    n_accepted += jd > 0;
    if ((iter + 1) % thin == 0 || (iter + 2) % n_sample_tau2 == 0) cur->sample_beta_sigma2(rng);
    tr.jump.push_back(jd);
    tr.mtype.push_back(move);
    tr.msize.push_back(movesize);
    if ((iter + 1) % thin == 0) {
      uint32_t nl = (uint32_t)cur->size();
      tr.msz.push_back(nl);
      tr.loci.insert(tr.loci.end(), cur->loci.begin(), cur->loci.end());
      if (use_types) tr.types.insert(tr.types.end(), cur->type_inds.begin(), cur->type_inds.end());
      tr.ll.push_back(cur->log_likelihood_);
      tr.lp.push_back(prior->compute_log_model(cur->Ns));
      tr.s2.push_back(cur->sigma2);
      if (save_beta) tr.beta.insert(tr.beta.end(), cur->beta.begin(), cur->beta.begin() + cur->blen);
      cur->compute_pve(pves);
      tr.pve.insert(tr.pve.end(), pves, pves + 3);
      tr.alpha.push_back(prior->alpha_);
    }
    if ((iter + 1) % n_rao == 0) {
      if (!flat_proposal_dist || n_rao_burnin <= 0) {
        dm->sample_missing(cur->model_inds, rng);
        p_raoblackwell(cur->y_hat, p_r.data(), use_types ? p_r_types.data() : nullptr);
      }
      if (n_rao_burnin <= 0) {
        double z1 = (double)(p_rao_n + 1), z2 = (double)p_rao_n / z1;
        for (size_t i = 0; i < m_g; ++i) p_rao[i] = z2 * p_rao[i] + p_r[i] / z1;
        if (use_types)
          for (size_t i = 0; i < m_g * n_types; ++i) p_rao_types[i] = z2 * p_rao_types[i] + p_r_types[i] / z1;
        ++p_rao_n;
      } else {
        n_rao_burnin--;
      }
      if (adaptation || n_rao_burnin > 0) {
        if (!flat_proposal_dist) {
          double z1 = (double)(p_proposal_n + 1), z2 = (double)p_proposal_n / z1;
          for (size_t i = 0; i < m_g; ++i) p_proposal[i] = z2 * p_proposal[i] + p_r[i] / z1;
          if (use_types)
            for (size_t i = 0; i < m_g * n_types; ++i)
              p_proposal_types[i] = z2 * p_proposal_types[i] + p_r_types[i] / z1;
        }
        if (adapt_p_move_size) {
          double t = std::max(1.0, k_move_size * (double)p_proposal_n);
          if (acpt_goal > 0) adapt_p_move_size_acptrate(2.0 + t);
          else adapt_p_move_size_jd_mb();
          geometric_dist_cdf(max_move_size, p_move_size, q_p_move_size.data());
        }
        ++p_proposal_n;
        if (!flat_proposal_dist) {
          compute_proposal_dist();
          for (size_t i = 0; i < m_g; ++i) q_rem[i] = std::max(1 - p_proposal[i], q_rem_min);
          dd_add->update_weights(q_add.data());
          dd_rem->update_weights(q_rem.data());
          if (use_types) compute_proposal_types_dist();
        }
      }
    }
  }

  void run(size_t k)
  {
    if (!started) start();
    size_t end = n_iter + k;
    for (size_t iter = n_iter; iter < end; ++iter) iterate(iter);
    n_iter = end;
  }
};

struct Port {
  bmg_options opt;
  std::vector<uint32_t> seeds;
  Data* data = nullptr;
  DataModel* dm0 = nullptr;
  PreXX* pre = nullptr;
  std::vector<Sampler*> chains;
  ~Port()
  {
    for (Sampler* s : chains) delete s;
    delete pre;
    delete dm0;
    delete data;
  }
};

}  // namespace bmgport_impl

using namespace bmgport_impl;

struct bmgport {
  Port p;
};

static void set_err(char* err, size_t len, const char* msg)
{
  if (err && len) { std::snprintf(err, len, "%s", msg); }
}

extern "C" int bmgport_create(const bmg_options* opt, const uint8_t* packed, const double* y,
                              const double* e, bmgport** out, char* err, size_t err_len)
{
  try {
    if (opt->sampler_type != 0) throw std::runtime_error("only the PMV sampler is restated");
    bmgport* P = new bmgport();
    P->p.opt = *opt;
    P->p.seeds.assign(opt->seeds, opt->seeds + opt->n_chains);
    P->p.opt.seeds = P->p.seeds.data();
    P->p.data = new Data(opt->n, opt->m_g, opt->m_e, packed, y, e, opt->recode_g_to_minor_allele_count != 0);
    std::vector<int> types(opt->types, opt->types + opt->n_types);
    P->p.dm0 = new DataModel(P->p.data, types);
    P->p.pre = new PreXX(P->p.dm0);
    for (uint32_t c = 0; c < opt->n_chains; ++c)
      P->p.chains.push_back(new Sampler(P->p.opt, P->p.data, P->p.pre, P->p.seeds[c]));
    *out = P;
    return 0;
  } catch (const std::exception& ex) {
    set_err(err, err_len, ex.what());
    return 1;
  }
}

extern "C" int bmgport_run(bmgport* P, uint64_t n_iter, uint32_t n_threads, const bmg_trace_sink* sink)
{
  std::vector<Sampler*>& ch = P->p.chains;
  std::vector<int> fail(ch.size(), 0);
  for (Sampler* s : ch) s->tr.clear();
  uint64_t iter0 = ch.empty() ? 0 : ch[0]->n_iter;
  auto work = [&](size_t c) {
    try { ch[c]->run(n_iter); } catch (...) { fail[c] = 1; }
  };
  if (n_threads <= 1 || ch.size() <= 1) {
    for (size_t c = 0; c < ch.size(); ++c) work(c);
  } else {
    size_t next = 0;
    while (next < ch.size()) {
      std::vector<std::thread> th;
      for (uint32_t t = 0; t < n_threads && next < ch.size(); ++t, ++next) th.emplace_back(work, next);
      for (auto& t : th) t.join();
    }
  }
  for (size_t c = 0; c < ch.size(); ++c) {
    if (fail[c]) return 1;
    if (sink && sink->fn) {
      Trace& t = ch[c]->tr;
      bmg_trace_chunk k;
      std::memset(&k, 0, sizeof(k));
      k.chain = (uint32_t)c;
      k.iter0 = iter0;
      k.n_iter = t.jump.size();
      k.jumpdistance = t.jump.data();
      k.move_type = t.mtype.data();
      k.move_size = t.msize.data();
      k.n_thin = t.msz.size();
      k.modelsize = t.msz.data();
      k.n_loci = t.loci.size();
      k.loci = t.loci.data();
      k.types = t.types.empty() ? nullptr : t.types.data();
      k.log_likelihood = t.ll.data();
      k.log_prior = t.lp.data();
      k.sigma2 = t.s2.data();
      k.alpha = t.alpha.data();
      k.pve = t.pve.data();
      k.n_beta = t.beta.size();
      k.beta = t.beta.empty() ? nullptr : t.beta.data();
      sink->fn(sink->user, &k);
    }
  }
  return 0;
}

extern "C" int bmgport_scan(bmgport* P, uint32_t chain, double* p_r, double* p_r_types)
{
  try {
    Sampler* s = P->p.chains.at(chain);
    std::vector<double> prt(s->use_types ? s->m_g * s->n_types : 1);
    s->p_raoblackwell(s->cur->y_hat, p_r, prt.data());
    if (p_r_types && s->use_types) std::memcpy(p_r_types, prt.data(), prt.size() * sizeof(double));
    return 0;
  } catch (...) {
    return 1;
  }
}

// the RB scan of the current state with the per-SNP log posterior odds of
// inclusion (the quantity the probabilities are the logistic of)
extern "C" int bmgport_scan_logodds(bmgport* P, uint32_t chain, double* logodds)
{
  try {
    Sampler* s = P->p.chains.at(chain);
    std::vector<double> pr(s->m_g), prt(s->use_types ? s->m_g * s->n_types : 1);
    s->logodds_out = logodds;
    s->p_raoblackwell(s->cur->y_hat, pr.data(), prt.data());
    s->logodds_out = nullptr;
    return 0;
  } catch (...) {
    return 1;
  }
}

extern "C" int bmgport_schur(bmgport* P, uint32_t chain, double* dlml, double* itv)
{
  try {
    P->p.chains.at(chain)->schur_scan(dlml, itv);
    return 0;
  } catch (...) {
    return 1;
  }
}

extern "C" int bmgport_scan_yhat(bmgport* P, uint32_t chain, const double* y_hat, double sigma2,
                                 double* p_r, double* p_r_types)
{
  try {
    Sampler* s = P->p.chains.at(chain);
    std::vector<double> yh(y_hat, y_hat + s->data->n);
    s->cur->sigma2 = sigma2;
    std::vector<double> prt(s->use_types ? s->m_g * s->n_types : 1);
    s->p_raoblackwell(yh, p_r, prt.data());
    if (p_r_types && s->use_types) std::memcpy(p_r_types, prt.data(), prt.size() * sizeof(double));
    return 0;
  } catch (...) {
    return 1;
  }
}

/* The log posterior odds of the same scan (the per-SNP Bayes factor with its
   prior odds, src/sampler.cpp:193-195) against the given y_hat and sigma2. */
extern "C" int bmgport_scan_yhat_logodds(bmgport* P, uint32_t chain, const double* y_hat, double sigma2,
                                         double* logodds)
{
  try {
    Sampler* s = P->p.chains.at(chain);
    std::vector<double> yh(y_hat, y_hat + s->data->n);
    s->cur->sigma2 = sigma2;
    std::vector<double> pr(s->m_g), prt(s->use_types ? s->m_g * s->n_types : 1);
    s->logodds_out = logodds;
    s->p_raoblackwell(yh, pr.data(), prt.data());
    s->logodds_out = nullptr;
    return 0;
  } catch (...) {
    return 1;
  }
}

extern "C" int bmgport_get_state(bmgport* P, uint32_t chain, bmg_chain_state* st, uint32_t* loci,
                                 uint8_t* type_inds, uint32_t cap)
{
  if (chain >= P->p.chains.size()) return 1;
  Sampler* s = P->p.chains[chain];
  st->model_size = (uint32_t)s->cur->size();
  st->log_likelihood = s->cur->log_likelihood_;
  st->log_prior = s->prior->compute_log_model(s->cur->Ns);
  st->sigma2 = s->cur->sigma2;
  st->alpha = s->prior->alpha_;
  st->n_iter = s->n_iter;
  st->n_accepted = s->n_accepted;
  st->p_move_size = s->p_move_size;
  st->rng_draws = s->rng.st.slot;
  for (uint32_t i = 0; i < st->model_size && i < cap; ++i) {
    if (loci) loci[i] = s->cur->loci[i];
    if (type_inds) type_inds[i] = s->cur->type_inds[i];
  }
  return 0;
}

/* The prior's shared 1/(tau2 alpha^2) per term type of a chain
   (Prior::get_inv_tau2_alpha2_value, src/prior.hpp:126-132): the precision every new
   term of that type gets while tau2 is shared. */
extern "C" int bmgport_get_inv_tau2_alpha2(bmgport* P, uint32_t chain, double* out4)
{
  if (chain >= P->p.chains.size()) return 1;
  for (int t = 0; t < 4; ++t) out4[t] = P->p.chains[chain]->prior->inv_tau2_alpha2[t];
  return 0;
}

extern "C" int bmgport_get_rao(bmgport* P, uint32_t chain, double* p_rao, double* p_rao_types)
{
  if (chain >= P->p.chains.size()) return 1;
  Sampler* s = P->p.chains[chain];
  std::memcpy(p_rao, s->p_rao.data(), s->m_g * sizeof(double));
  if (p_rao_types && s->use_types)
    std::memcpy(p_rao_types, s->p_rao_types.data(), s->p_rao_types.size() * sizeof(double));
  return 0;
}

extern "C" int bmgport_get_proposal(bmgport* P, uint32_t chain, double* p_prop, double* p_prop_types)
{
  if (chain >= P->p.chains.size()) return 1;
  Sampler* s = P->p.chains[chain];
  std::memcpy(p_prop, s->p_proposal.data(), s->m_g * sizeof(double));
  if (p_prop_types && s->use_types)
    std::memcpy(p_prop_types, s->p_proposal_types.data(), s->p_proposal_types.size() * sizeof(double));
  return 0;
}

extern "C" int bmgport_get_last_scan(bmgport* P, uint32_t chain, double* p_r, double* p_r_types)
{
  if (chain >= P->p.chains.size()) return 1;
  Sampler* s = P->p.chains[chain];
  std::memcpy(p_r, s->p_r.data(), s->m_g * sizeof(double));
  if (p_r_types && s->use_types) std::memcpy(p_r_types, s->p_r_types.data(), s->p_r_types.size() * sizeof(double));
  return 0;
}

extern "C" int bmgport_get_precomputed(bmgport* P, double* xx, uint32_t* offset)
{
  *offset = (uint32_t)P->p.pre->offset;
  if (xx) std::memcpy(xx, P->p.pre->xx.data(), P->p.pre->xx.size() * sizeof(double));
  return 0;
}

extern "C" int bmgport_get_data_stats(bmgport* P, double* out4)
{
  out4[0] = P->p.data->var_x;
  out4[1] = P->p.data->mean_x;
  out4[2] = P->p.data->var_y;
  out4[3] = P->p.data->yy;
  return 0;
}

extern "C" int bmgport_get_genotypes(bmgport* P, uint32_t type, uint64_t snp, double* out)
{
  if (snp >= P->p.data->m_g || type > 3) return 1;
  P->p.data->get_genotypes((int)type, snp, out);
  return 0;
}

extern "C" int bmgport_model_lml(bmgport* P, uint32_t n_add, const uint32_t* snps,
                                 const uint8_t* t_inds, const double* itv, double* lml)
{
  try {
    Sampler* s = P->p.chains.at(0);
    Stats st;
    Model m(P->p.data, s->dm, s->prior, &st, s->cur->cap);
    for (uint32_t i = 0; i < n_add; ++i) {
      m.add_term(snps[i], t_inds[i], &itv[2 * i]);
      lml[i] = m.log_likelihood_;
    }
    return 0;
  } catch (...) {
    return 1;
  }
}

/* The known-answer check of src/tests/model_tests.hpp:92-235: the model holds
   n_terms terms, of which the first const_loci stay; the exhaustive model
   set over the other m = n_terms - const_loci gives, per subset bit mask,
   the log likelihood plus the log prior change of adding that subset
   (exh_out), which must equal the same model built directly term by term
   (direct_out). */
extern "C" int bmgport_exh_modelset(bmgport* P, uint32_t n_terms, const uint32_t* snps,
                                    const uint8_t* t_inds, const double* itv, uint32_t const_loci,
                                    double* exh_out, double* direct_out)
{
  try {
    if (const_loci > n_terms || n_terms - const_loci > 16) return 1;
    Sampler* s = P->p.chains.at(0);
    Stats st;
    size_t cap = s->cur->cap;
    Model m(P->p.data, s->dm, s->prior, &st, cap);
    for (uint32_t i = 0; i < n_terms; ++i) m.add_term(snps[i], t_inds[i], &itv[2 * i]);
    ExhModel exh(P->p.data, s->dm, s->prior, &st, cap);
    exh.update_to_model(m, const_loci);
    size_t nm = n_terms - const_loci;
    double max_log_model;
    compute_exhaustive_modelset(nm, &exh, exh_out, max_log_model);
    for (size_t mask = 0; mask < ((size_t)1 << nm); ++mask) {
      Model d(P->p.data, s->dm, s->prior, &st, cap);
      int Ns[5] = {0, 0, 0, 0, 0};
      for (uint32_t i = 0; i < const_loci; ++i) {
        d.add_term(snps[i], t_inds[i], &itv[2 * i]);
        ++Ns[s->dm->types[t_inds[i]]];
      }
      int nl = (int)const_loci;
      double lp = 0;
      for (size_t j = 0; j < nm; ++j) {
        if (!((mask >> j) & 1)) continue;
        size_t k = const_loci + j;
        int type = s->dm->types[t_inds[k]];
        d.add_term(snps[k], t_inds[k], &itv[2 * k]);
        lp += s->prior->compute_log_change_on_add(Ns, nl, type);
        ++Ns[type];
        ++nl;
      }
      direct_out[mask] = lp + d.log_likelihood_;
    }
    return 0;
  } catch (...) {
    return 1;
  }
}

/* Log proposal probability of every sub-model of a delayed-rejection move
   (compute_proposal_probs_for_exh_modelset, src/sampler.cpp:980-1049), for
   the closed forms of src/tests/sampler_tests.hpp:611-700.  out (2^n_inds
   entries) is added to, as in the reference. */
extern "C" int bmgport_exh_proposal_probs(int use_types, int n_inds, const uint8_t* bit_to_normalized_order,
                                          const double* q_add, const double* q_rem, double z_add,
                                          double z_rem, uint64_t const_loci, uint64_t m_g,
                                          const double* log_q_add_types, double* out)
{
  if (n_inds < 1 || n_inds > 20) return 1;
  compute_proposal_probs_for_exh_modelset(use_types != 0, n_inds, bit_to_normalized_order, q_add, q_rem,
                                          z_add, z_rem, (size_t)const_loci, (size_t)m_g, log_q_add_types, out);
  return 0;
}

/* LML after adding n_add terms and then removing the term at model index
   rem (Model::remove_term, src/model.hpp:270-312: column shift, dchex job 2
   downdate of the Cholesky factor, sign fix and re-solve, src/model.hpp:508-556) */
extern "C" int bmgport_model_lml_remove(bmgport* P, uint32_t n_add, const uint32_t* snps,
                                        const uint8_t* t_inds, const double* itv, uint32_t rem, double* lml)
{
  try {
    if (rem >= n_add) return 1;
    Sampler* s = P->p.chains.at(0);
    Stats st;
    Model m(P->p.data, s->dm, s->prior, &st, s->cur->cap);
    for (uint32_t i = 0; i < n_add; ++i) m.add_term(snps[i], t_inds[i], &itv[2 * i]);
    m.remove_term((int)rem);
    *lml = m.log_likelihood_;
    return 0;
  } catch (...) {
    return 1;
  }
}

/* The proposal tree on its own (DiscreteDistribution, src/discrete_distribution.hpp:64-330),
   for the known answers of src/tests/discrete_distribution_tests.hpp.  ops
   are applied in order: op >= 0 zeroes SNP op (adddate), op < 0 restores SNP
   -op - 1 (remdate).  Then node values and the total are written, and
   n_samples draws (seed) are counted per SNP. */
extern "C" int bmgport_dd_exercise(const double* w, uint64_t n, const int64_t* ops, uint64_t n_ops,
                                   uint32_t seed, uint64_t n_samples, double* values_out, double* total_out,
                                   uint64_t* counts_out)
{
  try {
    if (n == 0) return 1;
    Rand rng(seed, 1.0);
    DD dd(w, (size_t)n, &rng);
    for (uint64_t i = 0; i < n_ops; ++i) {
      int64_t op = ops[i];
      if (op >= (int64_t)n || -op - 1 >= (int64_t)n) return 1;
      if (op >= 0) dd.adddate((size_t)op);
      else dd.remdate((size_t)(-op - 1));
    }
    if (values_out) for (uint64_t i = 0; i < n; ++i) values_out[i] = dd.value[i];
    *total_out = dd.total_w;
    if (counts_out) {
      for (uint64_t i = 0; i < n; ++i) counts_out[i] = 0;
      for (uint64_t i = 0; i < n_samples; ++i) {
        size_t k = dd.sample();
        if (k >= n) return 2;
        ++counts_out[k];
      }
    }
    return 0;
  } catch (...) {
    return 1;
  }
}

/* Missing-call imputation of one SNP (DataModel::sample_missing_single and
   update_prexx_cov, src/data_model.cpp:90-167), for the known answers of
   src/tests/data_model_tests.hpp:129-322: n_reps draws from the chain's
   stream, counting the value imputed for the SNP's first missing call; then
   the SNP's precomputed row corrected for the last draw (xx_out, offset
   values) and its four codings with the imputed values (geno_out, 4 x n). */
extern "C" int bmgport_missing_step(bmgport* P, uint32_t chain, uint64_t snp, uint64_t n_reps, double* xx_out,
                                    double* geno_out, uint64_t* counts)
{
  if (chain >= P->p.chains.size() || snp >= P->p.data->m_g) return 1;
  Sampler* s = P->p.chains[chain];
  for (int k = 0; k < 3; ++k) counts[k] = 0;
  for (uint64_t r = 0; r < n_reps && !s->dm->miss_val[snp].empty(); ++r) {
    s->dm->sample_missing_single((uint32_t)snp, s->rng);
    ++counts[(int)s->dm->miss_val[snp][0]];
  }
  const PreXX* pre = P->p.pre;
  for (int i = 0; i < pre->offset; ++i) xx_out[i] = pre->xx[snp * pre->offset + i];
  s->dm->update_prexx_cov(snp, xx_out);
  size_t n = P->p.data->n;
  for (int t = 0; t < 4; ++t) s->dm->get_genotypes(t, snp, geno_out + t * n);
  return 0;
}

/* Draws of (sigma2, beta) from their joint conditional posterior given a
   model of n_add terms (Model::sample_beta_sigma2, src/model.hpp:326-342,
   Rand::rand_mvnormal_invchol, src/rand.hpp:144-168), from a stream of its
   own (seed), for the distribution checks of
   src/tests/model_tests.hpp:314-410.  beta_out holds n_samples rows of
   *blen coefficients (constant first, then the model's columns). */
extern "C" int bmgport_sample_beta_sigma2(bmgport* P, uint32_t n_add, const uint32_t* snps, const uint8_t* t_inds,
                                          const double* itv, uint32_t seed, uint64_t n_samples, double* s2_out,
                                          double* beta_out, uint32_t blen_cap, uint32_t* blen)
{
  try {
    Sampler* s = P->p.chains.at(0);
    Stats st;
    Model m(P->p.data, s->dm, s->prior, &st, s->cur->cap);
    m.compute_log_likelihood();
    for (uint32_t i = 0; i < n_add; ++i) m.add_term(snps[i], t_inds[i], &itv[2 * i]);
    Rand rng(seed, s->prior->n_plus_nu);
    for (uint64_t r = 0; r < n_samples; ++r) {
      m.sample_beta_sigma2(rng);
      if (m.blen > blen_cap) return 1;
      s2_out[r] = m.sigma2;
      for (size_t j = 0; j < m.blen; ++j) beta_out[r * blen_cap + j] = m.beta[j];
    }
    *blen = (uint32_t)m.blen;
    return 0;
  } catch (...) {
    return 1;
  }
}

/* The model prior of chain 0 (Prior::compute_log_model and the changes on
   add, remove and type switch, src/prior.hpp:144-183): out = {log model
   prior of Ns, change on adding a term of type ta with nl loci, change on
   removing one of type ta with nl loci, change on switching ta -> tr}. */
extern "C" int bmgport_prior_terms(bmgport* P, const int32_t* Ns, int32_t nl, int32_t ta, int32_t tr, double* out)
{
  if (P->p.chains.empty() || ta < 0 || ta > 4 || tr < 0 || tr > 4) return 1;
  const Prior* pr = P->p.chains[0]->prior;
  int ns[5];
  for (int t = 0; t < 5; ++t) ns[t] = Ns[t];
  out[0] = pr->compute_log_model(ns);
  out[1] = pr->compute_log_change_on_add(ns, nl, ta);
  out[2] = pr->compute_log_change_on_rem(ns, nl, ta);
  out[3] = pr->compute_log_change_on_swi(ns, ta, tr);
  return 0;
}

extern "C" void bmgport_destroy(bmgport* P) { delete P; }
