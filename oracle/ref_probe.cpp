// ORACLE / TEST INFRASTRUCTURE, never linked into the product.
//
// Reads one INI file with the reference's own option parser
// (bmagwa::Options, src/options.hpp:138-321, built from the unmodified
// reference sources by oracle/Makefile) and prints every parsed field as
// "opt.<name>=<value>" lines, or "opt.error=<message>" when the parser
// throws.  With --data it also loads the data the INI names with the
// reference's Data class (src/data.hpp:45-72, src/data.cpp:141-434) and
// prints the phenotypes, the covariates and the summary statistics as
// "data.<name>=<value>" lines, or "data.error=<message>".
// tests/golden/make_golden.py runs it over the reference's INI files, over
// edited copies and over edited input files, to pin the product's parser
// (bmg_options_from_ini) and readers (bmg_read_plink).
#include <cstdio>
#include <exception>
#include <string>

#include "data.hpp"
#include "options.hpp"

static void put(const char* k, const std::string& v) { std::printf("opt.%s=%s\n", k, v.c_str()); }
static void put(const char* k, double v) { std::printf("opt.%s=%.17g\n", k, v); }
static void put(const char* k, unsigned long long v) { std::printf("opt.%s=%llu\n", k, v); }

int main(int argc, char** argv)
{
  bool data = argc == 3 && std::string(argv[1]) == "--data";
  if (argc != 2 && !data) {
    std::fprintf(stderr, "usage: ref_probe [--data] INIFILE\n");
    return 2;
  }
  try {
    bmagwa::Options o(argv[argc - 1]);
    if (data) {
      try {
        bmagwa::Data d(o.n, o.m_g, o.m_e, o.file_fam, o.file_g, o.recode_g_to_minor_allele_count, o.file_e,
                       o.file_y);
        for (size_t i = 0; i < o.n; ++i) std::printf("data.y.%zu=%.17g\n", i, d.y()(i));
        for (size_t j = 1; j < d.m_e; ++j)
          for (size_t i = 0; i < o.n; ++i) std::printf("data.e.%zu.%zu=%.17g\n", j - 1, i, d.e()(i, j));
        std::printf("data.yy=%.17g\ndata.var_y=%.17g\ndata.mean_x=%.17g\ndata.var_x=%.17g\n", d.yy(),
                    d.var_y(), d.mean_x(), d.var_x());
      } catch (const std::exception& ex) {
        std::printf("data.error=%s\n", ex.what());
      }
      return 0;
    }
    put("file_fam", o.file_fam);
    put("file_g", o.file_g);
    put("file_e", o.file_e);
    put("file_y", o.file_y);
    put("n", (unsigned long long)o.n);
    put("m_g", (unsigned long long)o.m_g);
    put("m_e", (unsigned long long)o.m_e);
    put("recode_g_to_minor_allele_count", (unsigned long long)o.recode_g_to_minor_allele_count);
    std::string types;
    for (size_t i = 0; i < o.types.size(); ++i) types += (i ? "," : "") + std::to_string((int)o.types[i]);
    put("types", types);
    put("sampler_type", (unsigned long long)o.sampler_type);
    put("do_n_iter", (unsigned long long)o.do_n_iter);
    put("n_rao", (unsigned long long)o.n_rao);
    put("n_rao_burnin", (unsigned long long)o.n_rao_burnin);
    put("thin", (unsigned long long)o.thin);
    put("n_sample_tau2_and_missing", (unsigned long long)o.n_sample_tau2_and_missing);
    put("max_move_size", (unsigned long long)o.max_move_size);
    put("max_SNP_neighborhood_size", (unsigned long long)o.max_SNP_neighborhood_size);
    put("p_move_size", o.p_move_size);
    put("p_move_size_nbs", o.p_move_size_nbs);
    put("p_move_size_nbc", o.p_move_size_nbc);
    put("adapt_p_move_size", (unsigned long long)o.adapt_p_move_size);
    put("p_move_size_acpt_goal", o.p_move_size_acpt_goal);
    put("adaptation", (unsigned long long)o.adaptation);
    put("flat_proposal_dist", (unsigned long long)o.flat_proposal_dist);
    put("save_beta", (unsigned long long)o.save_beta);
    put("verbosity", (unsigned long long)o.verbosity);
    put("delay_rejection", (unsigned long long)o.delay_rejection);
    put("basename", o.basename);
    put("n_chains", (unsigned long long)o.n_threads);
    std::string seeds;
    for (size_t i = 0; i < o.seeds.size(); ++i) seeds += (i ? "," : "") + std::to_string(o.seeds[i]);
    put("seeds", seeds);
    put("e_qg", o.e_qg);
    put("var_qg", o.var_qg);
    put("nu_sigma2", o.nu_sigma2);
    put("s2_sigma2", o.s2_sigma2);
    put("R2mode_sigma2", o.R2mode_sigma2);
    put("mu_alpha", o.mu_alpha);
    put("inv_tau2_e_const_val", o.inv_tau2_e_const_val);
    put("inv_tau2_e_val", o.inv_tau2_e_val);
    put("use_individual_tau2", (unsigned long long)o.use_individual_tau2);
    for (int t = 0; t < 5; ++t) put(("types_prior." + std::to_string(t)).c_str(), o.types_prior[t]);
    for (int t = 0; t < 4; ++t) {
      put(("nu_tau2." + std::to_string(t)).c_str(), o.nu_tau2[t]);
      put(("s2_tau2." + std::to_string(t)).c_str(), o.s2_tau2[t]);
      put(("eh_tau2." + std::to_string(t)).c_str(), o.eh_tau2[t]);
    }
  } catch (const std::exception& ex) {
    put("error", std::string(ex.what()));
  }
  return 0;
}
