/*
 * Stand-in for <boost/lexical_cast.hpp>; the reference only converts a chain
 * index to a string (src/options.hpp:119).  ORACLE / TEST INFRASTRUCTURE.
 */
#ifndef BMG_SHIM_BOOST_LEXICAL_CAST_HPP_
#define BMG_SHIM_BOOST_LEXICAL_CAST_HPP_

#include <sstream>
#include <string>

namespace boost {

template <class Target, class Source>
Target lexical_cast(const Source& s)
{
  std::ostringstream os;
  os << s;
  return os.str();
}

}  // namespace boost

#endif
