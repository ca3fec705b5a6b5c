// INI parsing and option semantics of the reference CLI, for libbmg.
//
// The INI reader follows the grammar of the inih parser the reference vendors
// (src/inih/ini.c:57-130): ';' or '#' comment lines, "[section]", "name = value"
// or "name : value", an inline ';' comment when preceded by whitespace,
// continuation lines with leading whitespace, keys looked up case-insensitively
// as "section.name" (src/inih/cpp/INIReader.cpp:35-45), later keys win.
// The option rules, defaults, warnings and error messages follow
// bmagwa::Options::parse_options (src/options.hpp:138-321).
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "bmg.h"

namespace bmg_host {

class IniFile {
 public:
  explicit IniFile(const std::string& path) : error_(0)
  {
    std::FILE* f = std::fopen(path.c_str(), "r");
    if (!f) { error_ = -1; return; }
    char buf[200];  /* the reference reads lines of at most 199 characters */
    std::string section, prev;
    int lineno = 0;
    while (std::fgets(buf, sizeof(buf), f)) {
      ++lineno;
      std::string line(buf);
      rstrip(line);
      size_t lead = 0;
      while (lead < line.size() && std::isspace((unsigned char)line[lead])) ++lead;
      std::string start = line.substr(lead);
      if (!prev.empty() && !start.empty() && lead > 0) {
        values_[key(section, prev)] = start;  /* continuation line */
      } else if (!start.empty() && (start[0] == ';' || start[0] == '#')) {
        /* comment */
      } else if (!start.empty() && start[0] == '[') {
        size_t e = find_char_or_comment(start, 1, ']');
        if (e < start.size() && start[e] == ']') {
          section = start.substr(1, e - 1);
          prev.clear();
        } else if (!error_) {
          error_ = lineno;
        }
      } else if (!start.empty()) {
        size_t e = find_char_or_comment(start, 0, '=');
        if (e >= start.size() || start[e] != '=') e = find_char_or_comment(start, 0, ':');
        if (e < start.size() && (start[e] == '=' || start[e] == ':')) {
          std::string name = start.substr(0, e);
          rstrip(name);
          std::string value = start.substr(e + 1);
          size_t vb = 0;
          while (vb < value.size() && std::isspace((unsigned char)value[vb])) ++vb;
          value = value.substr(vb);
          size_t ve = find_char_or_comment(value, 0, '\0');
          value = value.substr(0, ve);
          rstrip(value);
          prev = name;
          values_[key(section, name)] = value;
        } else if (!error_) {
          error_ = lineno;
        }
      }
    }
    std::fclose(f);
  }
  int error() const { return error_; }
  std::string get(const std::string& s, const std::string& n, const std::string& def) const
  {
    std::map<std::string, std::string>::const_iterator it = values_.find(key(s, n));
    return it == values_.end() ? def : it->second;
  }

 private:
  int error_;
  std::map<std::string, std::string> values_;
  static void rstrip(std::string& s)
  {
    while (!s.empty() && std::isspace((unsigned char)s.back())) s.pop_back();
  }
  static size_t find_char_or_comment(const std::string& s, size_t from, char c)
  {
    bool ws = false;
    size_t i = from;
    while (i < s.size() && s[i] != c && !(ws && s[i] == ';')) {
      ws = std::isspace((unsigned char)s[i]) != 0;
      ++i;
    }
    return i;
  }
  static std::string key(const std::string& s, const std::string& n)
  {
    std::string k = s + "." + n;
    for (size_t i = 0; i < k.size(); ++i) k[i] = (char)std::tolower((unsigned char)k[i]);
    return k;
  }
};

class OptionParser {
 public:
  OptionParser(const IniFile& r, bool quiet) : r_(r), quiet_(quiet) {}

  std::string str(const char* s, const char* n, bool allow_default, const std::string& def)
  {
    std::string res = r_.get(s, n, "DEFAULT_VALUE");
    bool none = res.empty() || res == "DEFAULT_VALUE";
    if (none && !allow_default)
      throw std::runtime_error(std::string("Cannot leave option empty: ") + s + "." + n);
    if (none) {
      warn(def, s, n);
      return def;
    }
    return res;
  }
  double dbl(const char* s, const char* n, bool allow_default, double def)
  {
    std::string res = r_.get(s, n, "DEFAULT_VALUE");
    bool none = res.empty() || res == "DEFAULT_VALUE";
    if (none && !allow_default)
      throw std::runtime_error(std::string("Cannot leave option empty: ") + s + "." + n);
    if (none) {
      std::ostringstream os;
      os << def;
      warn(os.str(), s, n);
      return def;
    }
    return convert<double>(res);
  }
  double dbl01(const char* s, const char* n, bool ad, double def)
  {
    double v = dbl(s, n, ad, def);
    if (v < 0 || v > 1) throw std::runtime_error("Value in 0..1 required");
    return v;
  }
  double dblpos(const char* s, const char* n, bool ad, double def)
  {
    double v = dbl(s, n, ad, def);
    if (v <= 0) throw std::runtime_error(std::string("Positive value required for ") + s + "." + n);
    return v;
  }
  double dblnonneg(const char* s, const char* n, bool ad, double def)
  {
    double v = dbl(s, n, ad, def);
    if (v < 0) throw std::runtime_error(std::string("Non-negative value required for ") + s + "." + n);
    return v;
  }
  int integer(const char* s, const char* n, bool allow_default, int def)
  {
    std::string res = r_.get(s, n, "DEFAULT_VALUE");
    bool none = res.empty() || res == "DEFAULT_VALUE";
    if (none && !allow_default)
      throw std::runtime_error(std::string("Cannot leave option empty: ") + s + "." + n);
    if (none) {
      warn(std::to_string(def), s, n);
      return def;
    }
    return convert<int>(res);
  }
  int intnonneg(const char* s, const char* n, bool ad, int def)
  {
    int v = integer(s, n, ad, def);
    if (v < 0) throw std::runtime_error("Nonnegative integer required");
    return v;
  }
  int intpos(const char* s, const char* n, bool ad, int def)
  {
    int v = integer(s, n, ad, def);
    if (v <= 0) throw std::runtime_error("Positive integer required");
    return v;
  }
  bool boolean(const char* s, const char* n, bool ad, int def)
  {
    int v = integer(s, n, ad, def);
    if (v != 0 && v != 1) throw std::runtime_error("Boolean value required (0 or 1)");
    return v == 1;
  }
  template <class T>
  static T convert(const std::string& s)
  {
    std::istringstream is(s);
    T x;
    char c;
    if (!(is >> x) || is.get(c)) throw std::runtime_error("Invalid conversion.");
    return x;
  }

 private:
  const IniFile& r_;
  bool quiet_;
  void warn(const std::string& def, const char* s, const char* n)
  {
    if (!quiet_)
      std::cout << "Warning: using default value of " << def << " for option " << s << "." << n
                << std::endl;
  }
};

static std::vector<std::string> split_trim(const std::string& in)
{
  std::vector<std::string> out;
  std::string cur;
  for (size_t i = 0; i <= in.size(); ++i) {
    if (i == in.size() || in[i] == ',') {
      size_t b = 0, e = cur.size();
      while (b < e && std::isspace((unsigned char)cur[b])) ++b;
      while (e > b && std::isspace((unsigned char)cur[e - 1])) --e;
      out.push_back(cur.substr(b, e - b));
      cur.clear();
    } else {
      cur += in[i];
    }
  }
  return out;
}

static void copy_path(char* dst, const std::string& src)
{
  if (src.size() >= BMG_MAX_PATH) throw std::runtime_error("path longer than BMG_MAX_PATH");
  std::memcpy(dst, src.c_str(), src.size() + 1);
}

}  // namespace bmg_host

using namespace bmg_host;

extern "C" size_t bmg_options_size(void) { return sizeof(bmg_options); }

extern "C" bmg_status bmg_options_default(bmg_options* o)
{
  if (!o) return BMG_EINVAL;
  std::memset(o, 0, sizeof(*o));
  o->sampler_type = 0;
  o->max_move_size = 20;
  o->max_SNP_neighborhood_size = 10;
  o->p_move_size = 0.2;
  o->p_move_size_nbs = 0.2;
  o->p_move_size_nbc = 0.2;
  o->adapt_p_move_size = 1;
  o->p_move_size_acpt_goal = 0.0;
  std::snprintf(o->basename, BMG_MAX_PATH, "chain");
  o->n_chains = 1;
  o->R2mode_sigma2 = 0.0;
  o->s2_sigma2 = 0.0;
  o->mu_alpha = 0.0;
  o->inv_tau2_e_val = 0.0;
  for (int t = 0; t < 5; ++t) o->types_prior[t] = 1.0;
  o->max_model_size = 1024;
  o->scan_limbs = 6;
  o->scan_impl = BMG_SCAN_TCGEN05;
  o->proposal = BMG_PROPOSAL_ADAPTIVE;
  o->graph_iters = 64;
  o->write_files = 0;
  o->quiet = 0;
  o->learned_mix = 0.3;
  o->learned_topk = 1024;
  o->learned_every = 10;
  o->learned_steps = 4;
  o->learned_lr = 1e-3;
  return BMG_OK;
}

extern "C" bmg_status bmg_options_from_ini(const char* path, bmg_options* o, uint32_t* seeds_buf,
                                           uint32_t seeds_cap, char* err, size_t err_len)
{
  try {
    if (!path || !o) throw std::runtime_error("null argument");
    int quiet = o->quiet;
    bmg_options_default(o);
    o->quiet = quiet;
    IniFile r(path);
    if (r.error() != 0) throw std::runtime_error("Cannot load/parse configuration file.");
    OptionParser p(r, quiet != 0);
    /* src/options.hpp:140-321, same order */
    o->n = (uint64_t)p.intpos("sizes", "n", false, 0);
    o->m_g = (uint64_t)p.intpos("sizes", "m_g", false, 0);
    o->m_e = (uint32_t)p.intnonneg("sizes", "m_e", true, 0);
    copy_path(o->file_fam, p.str("datafiles", "file_fam", false, ""));
    copy_path(o->file_g, p.str("datafiles", "file_g", false, ""));
    copy_path(o->file_e, p.str("datafiles", "file_e", o->m_e == 0, ""));
    copy_path(o->file_y, p.str("datafiles", "file_y", true, ""));
    o->recode_g_to_minor_allele_count = p.boolean("datafiles", "recode_g_to_minor_allele_count", true, 0);
    std::string types_str = p.str("model", "types", false, "");
    std::string sampler_type = p.str("sampler", "type", true, "PMV");
    o->do_n_iter = (uint64_t)p.intpos("sampler", "do_n_iter", false, 0);
    o->n_rao = (uint64_t)p.intnonneg("sampler", "n_rao", false, 0);
    o->n_rao_burnin = (uint64_t)p.intnonneg("sampler", "n_rao_burnin", false, 0);
    o->thin = (uint64_t)p.intpos("sampler", "thin", false, 0);
    o->n_sample_tau2_and_missing = (uint64_t)p.intpos("sampler", "n_sample_tau2_and_missing", false, 0);
    o->max_move_size = (uint32_t)p.intpos("sampler", "max_move_size", true, 20);
    o->max_SNP_neighborhood_size = (uint32_t)p.intpos("sampler", "max_SNP_neighborhood_size", true, 10);
    o->p_move_size = p.dblpos("sampler", "p_move_size", true, 0.2);
    if (o->p_move_size > 1) throw std::runtime_error("Config error: p_move_size must be <= 1.");
    o->p_move_size_nbs = p.dblpos("sampler", "p_move_size_nbs", true, 0.2);
    if (o->p_move_size_nbs > 1) throw std::runtime_error("Config error: p_move_size_nbs must be <= 1.");
    o->p_move_size_nbc = p.dblpos("sampler", "p_move_size_nbc", true, 0.2);
    if (o->p_move_size_nbc > 1) throw std::runtime_error("Config error: p_move_size_nbc must be <= 1.");
    o->adapt_p_move_size = p.boolean("sampler", "adapt_p_move_size", true, 1);
    o->p_move_size_acpt_goal = p.dblnonneg("sampler", "p_move_size_acpt_goal", true, 0.0);
    if (o->p_move_size_acpt_goal > 1)
      throw std::runtime_error("Config error: p_move_size_acpt_goal must be <= 1.");
    o->adaptation = p.boolean("sampler", "adaptation", true, 0);
    o->flat_proposal_dist = p.boolean("sampler", "flat_proposal_dist", true, 0);
    o->save_beta = p.boolean("sampler", "save_beta", true, 0);
    o->verbosity = (uint64_t)p.intnonneg("sampler", "verbosity", false, 0);
    o->delay_rejection = (uint32_t)p.intnonneg("sampler", "delay_rejection", true, 0);
    copy_path(o->basename, p.str("thread", "basename", true, "chain"));
    o->n_chains = (uint32_t)p.intpos("thread", "n_threads", true, 1);
    std::string seeds_str = p.str("thread", "seeds", false, "");
    o->e_qg = p.dblpos("prior", "e_qg", false, 0.0);
    o->var_qg = p.dblpos("prior", "var_qg", false, 0.0);
    o->nu_sigma2 = p.dblpos("prior", "nu_sigma2", false, 0.0);
    o->R2mode_sigma2 = p.dbl01("prior", "R2mode_sigma2", true, 0.0);
    o->s2_sigma2 = p.dblnonneg("prior", "s2_sigma2", true, 0.0);
    if (o->s2_sigma2 <= 0 && o->R2mode_sigma2 <= 0)
      throw std::runtime_error("Config error: s2_sigma2 or R2mode_sigma2 must be > 0.");
    o->mu_alpha = p.dbl("prior", "mu_alpha", true, 0.0);
    o->inv_tau2_e_const_val = p.dblnonneg("prior", "inv_tau2_e_const_val", false, 0.0);
    o->inv_tau2_e_val = p.dblnonneg("prior", "inv_tau2_e_val", o->m_e == 0, 0.0);
    o->use_individual_tau2 = p.boolean("prior", "use_individual_tau2", true, 0);
    o->types_prior[BMG_TYPE_A] = p.dbl("prior", "type_A", true, 1.0);
    o->types_prior[BMG_TYPE_H] = p.dbl("prior", "type_H", true, 1.0);
    o->types_prior[BMG_TYPE_R] = p.dbl("prior", "type_R", true, 1.0);
    o->types_prior[BMG_TYPE_D] = p.dbl("prior", "type_D", true, 1.0);
    o->types_prior[BMG_TYPE_AH] = p.dbl("prior", "type_AH", true, 1.0);
    if (sampler_type == "PMV") o->sampler_type = 0;
    else if (sampler_type == "NK") o->sampler_type = 1;
    else if (sampler_type == "KSC") o->sampler_type = 2;
    else if (sampler_type == "G") o->sampler_type = 3;
    else throw std::runtime_error("Config error: unknown sampler type");
    if (o->n_rao % o->thin != 0) throw std::runtime_error("Config error: n_rao should be a multiple of thin");
    std::vector<int> types;
    for (const std::string& t : split_trim(types_str)) {
      if (t == "A") types.push_back(BMG_TYPE_A);
      else if (t == "H") types.push_back(BMG_TYPE_H);
      else if (t == "D") types.push_back(BMG_TYPE_D);
      else if (t == "R") types.push_back(BMG_TYPE_R);
      else if (t == "AH") types.push_back(BMG_TYPE_AH);
      else throw std::runtime_error("Config error: Unknown model type");
    }
    std::sort(types.begin(), types.end());
    if (types.empty()) throw std::runtime_error("Config error: Types cannot be empty");
    if (types.size() > 5) throw std::runtime_error("Config error: too many types");
    if (o->sampler_type != 0 && (types.size() != 1 || types[0] != BMG_TYPE_A))
      throw std::runtime_error("Config error: NK/KSC/G samplers support only A effect types");
    o->n_types = (uint32_t)types.size();
    for (size_t i = 0; i < types.size(); ++i) o->types[i] = types[i];
    auto has = [&](int t) { return std::find(types.begin(), types.end(), t) != types.end(); };
    const char* nu_k[4] = {"nu_tau2_A", "nu_tau2_H", "nu_tau2_D", "nu_tau2_R"};
    const char* eh_k[4] = {"eh_tau2_A", "eh_tau2_H", "eh_tau2_D", "eh_tau2_R"};
    const char* s2_k[4] = {"s2_tau2_A", "s2_tau2_H", "s2_tau2_D", "s2_tau2_R"};
    const char* names[4] = {"A", "H", "D", "R"};
    for (int t = 0; t < 4; ++t) {
      bool need = has(t) || ((t == BMG_TYPE_A || t == BMG_TYPE_H) && has(BMG_TYPE_AH));
      if (!need) continue;
      o->nu_tau2[t] = p.dblpos("prior", nu_k[t], false, 0.0);
      o->eh_tau2[t] = p.dbl01("prior", eh_k[t], true, 0.0);
      o->s2_tau2[t] = p.dblnonneg("prior", s2_k[t], true, 0.0);
      if (o->s2_tau2[t] <= 0 && o->eh_tau2[t] <= 0)
        throw std::runtime_error(std::string("Config error: s2_tau2_") + names[t] + " or eh_tau2_" +
                                 names[t] + " must be > 0.");
    }
    std::vector<uint32_t> seeds;
    for (const std::string& s : split_trim(seeds_str)) seeds.push_back(OptionParser::convert<uint32_t>(s));
    if (seeds.size() != o->n_chains)
      throw std::runtime_error("Config error: Number of seeds must equal n_threads");
    for (size_t i = 0; i + 1 < seeds.size(); ++i)
      for (size_t j = i + 1; j < seeds.size(); ++j)
        if (seeds[i] == seeds[j]) throw std::runtime_error("Seeds are not unique");
    if (seeds.size() > seeds_cap) throw std::runtime_error("seeds buffer too small");
    for (size_t i = 0; i < seeds.size(); ++i) seeds_buf[i] = seeds[i];
    o->seeds = seeds_buf;
    return BMG_OK;
  } catch (const std::exception& ex) {
    if (err && err_len) std::snprintf(err, err_len, "%s", ex.what());
    return BMG_EINVAL;
  }
}
