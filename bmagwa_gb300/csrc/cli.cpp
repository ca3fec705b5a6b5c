// bmagwa-gb300 INIFILE: the command-line entry of the reference
// (`bmagwa INIFILE`, src/main.cpp:36-120) on the GB300 path.
//
// Same input (a reference INI file and the PLINK files it names) and the same
// outputs (the binary trace files of every chain, the log, prior and sampler
// statistics files), written by libbmg.  All chains run in one context on the
// current CUDA device instead of one host thread per chain.  Options the GPU
// path does not run (another sampler type, delayed rejection, missing calls)
// stop the program with the library's message before any sampling.
#include <cstdio>
#include <cstring>
#include <vector>

#include "bmg.h"

namespace {

int fail(const char* what, const char* msg)
{
  std::fprintf(stderr, "bmagwa-gb300: %s: %s\n", what, msg);
  return 1;
}

// ctx NULL: the failed call was bmg_create, whose message the library keeps
// per thread
int fail_ctx(bmg_ctx* ctx, const char* what, bmg_status st)
{
  const char* msg = bmg_last_error(ctx);
  std::fprintf(stderr, "bmagwa-gb300: %s: %s%s%s\n", what, bmg_status_string(st), msg && *msg ? ": " : "",
               msg ? msg : "");
  if (ctx) bmg_destroy(ctx);
  return 1;
}

}  // namespace

int main(int argc, char** argv)
{
  std::printf("bmagwa-gb300: BMAGWA MCMC over SNP inclusion on a GB300 GPU\n\n");
  std::fflush(stdout);
  if (argc != 2) {
    std::printf("Usage: %s INIFILE\n", argv[0]);
    return 0;
  }
  bmg_options opt;
  bmg_options_default(&opt);
  opt.quiet = 0;
  static uint32_t seeds[1 << 16];
  char err[1024] = {0};
  if (bmg_options_from_ini(argv[1], &opt, seeds, (uint32_t)(sizeof(seeds) / sizeof(seeds[0])), err, sizeof(err)) !=
      BMG_OK)
    return fail("options", err);
  opt.quiet = 0;
  opt.write_files = 1;

  const uint64_t n = opt.n, p = opt.m_g;
  std::vector<uint8_t> packed((size_t)(p * ((n + 3) / 4)));
  std::vector<double> y((size_t)n), e((size_t)(n * opt.m_e));
  if (bmg_read_plink(&opt, packed.data(), y.data(), opt.m_e ? e.data() : nullptr, err, sizeof(err)) != BMG_OK)
    return fail("data", err);

  bmg_ctx* ctx = nullptr;
  bmg_status st = bmg_create(&opt, &ctx);
  if (st != BMG_OK) return fail_ctx(ctx, "create", st);
  if ((st = bmg_load_bed(ctx, packed.data(), n, p)) != BMG_OK) return fail_ctx(ctx, "load_bed", st);
  std::vector<uint8_t>().swap(packed);
  if ((st = bmg_set_phenotypes(ctx, y.data(), nullptr, 1)) != BMG_OK) return fail_ctx(ctx, "phenotypes", st);
  if ((st = bmg_set_covariates(ctx, opt.m_e ? e.data() : nullptr, opt.m_e)) != BMG_OK)
    return fail_ctx(ctx, "covariates", st);
  if ((st = bmg_precompute(ctx)) != BMG_OK) return fail_ctx(ctx, "precompute", st);
  std::printf("Sampling %llu iterations of %u chains\n", (unsigned long long)opt.do_n_iter, opt.n_chains);
  std::fflush(stdout);
  if ((st = bmg_run(ctx, opt.do_n_iter, nullptr)) != BMG_OK) return fail_ctx(ctx, "run", st);
  if ((st = bmg_finish(ctx)) != BMG_OK) return fail_ctx(ctx, "finish", st);
  bmg_destroy(ctx);
  std::printf("Done: trace files written under basename %s\n", opt.basename);
  return 0;
}
