// PLINK readers for libbmg: .fam (phenotype), alternate phenotype and
// covariate files, and the SNP-major .bed payload.  Row matching, the
// acceptance rules and the error messages follow bmagwa::Data::read_fam /
// read_y / read_e / read_g (src/data.cpp:141-273).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "bmg.h"
#include "bmg_internal.h"

namespace bmg_host {

typedef std::map<std::pair<std::string, std::string>, size_t> FamMap;

/* src/data.cpp:141-169 */
static void read_fam(const std::string& path, size_t n, double* y, FamMap& fam)
{
  std::ifstream file(path.c_str());
  size_t i = 0;
  while (file.good()) {
    std::string fid, iid, tmp;
    double v = NAN;
    file >> fid >> iid >> tmp >> tmp >> tmp >> v;
    if (file.good() && !fid.empty() && !iid.empty() && !std::isnan(v)) {
      if (i < n) y[i] = v;
      fam[std::make_pair(fid, iid)] = i;
      ++i;
    }
  }
  if (i != n || fam.size() != n) throw std::runtime_error("FAM file size does not match given n");
}

/* src/data.cpp:171-200 */
static void read_y(const std::string& path, size_t n, double* y, const FamMap& fam)
{
  std::ifstream file(path.c_str());
  size_t i = 0;
  while (file.good()) {
    std::string fid, iid;
    double v = NAN;
    file >> fid >> iid >> v;
    if (file.good() && !fid.empty() && !iid.empty() && !std::isnan(v)) {
      FamMap::const_iterator it = fam.find(std::make_pair(fid, iid));
      if (it != fam.end()) {
        y[it->second] = v;
        ++i;
      }
    }
  }
  if (i != n) throw std::runtime_error("Alternate phenotype file does not contain all phenotypes");
}

/* src/data.cpp:202-243; e is n x m_e column-major without the constant */
static void read_e(const std::string& path, size_t n, size_t m_e, double* e, const FamMap& fam)
{
  std::ifstream file(path.c_str());
  size_t i = 0;
  while (file.good()) {
    std::string fid, iid;
    std::vector<double> row(m_e, NAN);
    file >> fid >> iid;
    for (size_t j = 0; j < m_e; ++j) file >> row[j];
    if (file.good() && !fid.empty() && !iid.empty()) {
      bool nans = false;
      for (size_t j = 0; j < m_e; ++j) nans = nans || std::isnan(row[j]);
      if (nans) continue;
      FamMap::const_iterator it = fam.find(std::make_pair(fid, iid));
      if (it != fam.end()) {
        for (size_t j = 0; j < m_e; ++j) e[j * n + it->second] = row[j];
        ++i;
      }
    }
  }
  if (i != n) throw std::runtime_error("Covariate file does not contain all covariates");
}

/* src/data.cpp:245-273 */
static void read_bed(const std::string& path, size_t n, size_t m_g, uint8_t* packed)
{
  std::ifstream file(path.c_str(), std::ios::in | std::ios::binary);
  if (!file.good()) throw bmg_error(BMG_EIO, "BED file could not be opened");
  char b = 0;
  file.read(&b, 1);
  if (b != 0x6C) throw bmg_error(BMG_EIO, "BED file not recognised (magic number does not match)");
  file.read(&b, 1);
  if (b != 0x1B) throw bmg_error(BMG_EIO, "BED file not recognised (magic number does not match)");
  file.read(&b, 1);
  if (b != 0x01) throw bmg_error(BMG_EIO, "BED file not in snp-major format");
  size_t len = ((n + 3) / 4) * m_g;
  file.read(reinterpret_cast<char*>(packed), (std::streamsize)len);
  if (!file.good() || (size_t)file.gcount() != len) throw bmg_error(BMG_EIO, "Reading the BED file failed");
}

}  // namespace bmg_host

using namespace bmg_host;

extern "C" bmg_status bmg_read_plink(const bmg_options* o, uint8_t* packed, double* y, double* e,
                                     char* err, size_t err_len)
{
  try {
    if (!o || !packed || !y) throw bmg_error(BMG_EINVAL, "null argument");
    if (o->m_e > 0 && !e) throw bmg_error(BMG_EINVAL, "covariate buffer required when m_e > 0");
    FamMap fam;
    read_fam(o->file_fam, o->n, y, fam);
    if (o->file_y[0]) read_y(o->file_y, o->n, y, fam);
    if (o->m_e > 0) read_e(o->file_e, o->n, o->m_e, e, fam);
    read_bed(o->file_g, o->n, o->m_g, packed);
    return BMG_OK;
  } catch (const bmg_error& ex) {
    if (err && err_len) std::snprintf(err, err_len, "%s", ex.what());
    return ex.status;
  } catch (const std::exception& ex) {
    if (err && err_len) std::snprintf(err, err_len, "%s", ex.what());
    return BMG_EIO;
  }
}
