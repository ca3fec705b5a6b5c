/*
 * Stand-in for <boost/random.hpp> used only to compile the reference sources
 * as a test oracle (src/rand.hpp:26,174-186 are the only users).
 *
 * ORACLE / TEST INFRASTRUCTURE.  The engine named mt19937 here is NOT the
 * Mersenne twister: it is the counter-based stream of include/bmg_rng.h, so
 * that the compiled reference and the GPU sampler consume the same numbers.
 * uniform_01 / normal_distribution / gamma_distribution map to that header's
 * uniform, Box-Muller normal and Marsaglia-Tsang gamma draws.
 */
#ifndef BMG_SHIM_BOOST_RANDOM_HPP_
#define BMG_SHIM_BOOST_RANDOM_HPP_

#include <stdint.h>
#include "bmg_rng.h"

namespace boost {

class mt19937 {
 public:
  typedef uint32_t result_type;
  explicit mt19937(uint32_t seed) { bmg_rng_init(&state, seed); }
  bmg_rng_t state;
};

template <class RealType = double>
class uniform_01 {
 public:
  typedef RealType result_type;
  result_type operator()(mt19937& eng) const { return bmg_uniform01(&eng.state); }
};

template <class RealType = double>
class normal_distribution {
 public:
  typedef RealType result_type;
  explicit normal_distribution(RealType mean = 0, RealType sd = 1)
  : mean_(mean), sd_(sd) {}
  result_type operator()(mt19937& eng) const
  {
    return mean_ + sd_ * bmg_normal(&eng.state);
  }
 private:
  RealType mean_, sd_;
};

template <class RealType = double>
class gamma_distribution {
 public:
  typedef RealType result_type;
  explicit gamma_distribution(RealType alpha = 1) : alpha_(alpha) {}
  result_type operator()(mt19937& eng) const
  {
    return bmg_gamma(&eng.state, alpha_);
  }
 private:
  RealType alpha_;
};

template <class Engine, class Distribution>
class variate_generator {
 public:
  typedef typename Distribution::result_type result_type;
  variate_generator(Engine e, Distribution d) : eng_(e), dist_(d) {}
  result_type operator()() { return dist_(eng_); }
 private:
  Engine eng_;
  Distribution dist_;
};

}  // namespace boost

#endif
