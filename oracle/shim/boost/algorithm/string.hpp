/*
 * Stand-in for <boost/algorithm/string.hpp> (split, trim, is_any_of) used only
 * to compile the reference's option parser (src/options.hpp:236-301) as a test
 * oracle.  ORACLE / TEST INFRASTRUCTURE.
 */
#ifndef BMG_SHIM_BOOST_ALGO_STRING_HPP_
#define BMG_SHIM_BOOST_ALGO_STRING_HPP_

#include <string>
#include <vector>
#include <cctype>

namespace boost {

struct bmg_any_of_pred {
  std::string chars;
  bool operator()(char c) const { return chars.find(c) != std::string::npos; }
};

inline bmg_any_of_pred is_any_of(const std::string& chars)
{
  bmg_any_of_pred p;
  p.chars = chars;
  return p;
}

inline std::vector<std::string>& split(std::vector<std::string>& out,
                                       const std::string& in,
                                       const bmg_any_of_pred& pred)
{
  out.clear();
  std::string cur;
  for (size_t i = 0; i < in.size(); ++i) {
    if (pred(in[i])) {
      out.push_back(cur);
      cur.clear();
    } else {
      cur += in[i];
    }
  }
  out.push_back(cur);
  return out;
}

inline void trim(std::string& s)
{
  size_t b = 0, e = s.size();
  while (b < e && std::isspace((unsigned char)s[b])) ++b;
  while (e > b && std::isspace((unsigned char)s[e - 1])) --e;
  s = s.substr(b, e - b);
}

}  // namespace boost

#endif
