// Internal declarations shared by the host translation units of libbmg.
#ifndef BMG_INTERNAL_H_
#define BMG_INTERNAL_H_

#include <stdexcept>
#include <string>

#include "bmg.h"

namespace bmg_host {

// An error that carries the status the C ABI returns.
struct bmg_error : public std::runtime_error {
  bmg_status status;
  bmg_error(bmg_status s, const std::string& msg) : std::runtime_error(msg), status(s) {}
};

// Message returned by bmg_last_error(NULL) on the calling thread: set by the
// entry points that fail without a context (bmg_create,
// bmg_precompute_noalloc).
void set_thread_error(const std::string& msg);

}  // namespace bmg_host

#endif
