// Every extern "C" entry point of the library is a function-try-block
// closed by TBSLA_API_CATCH, so no C++ exception crosses the C ABI: a host
// allocation that fails (std::bad_alloc, or a std::vector asked for more
// than it can hold) returns TBSLA_ERR_ALLOC, any other exception
// TBSLA_ERR_INVALID_ARG.  The calls that replace a matrix's arrays (the
// setters, push_back, the generators, read) close with
// TBSLA_API_CATCH_EMPTY(m) instead: a matrix whose arrays were being
// rebuilt when the exception came is left empty, as after
// tbsla_matrix_create, never with arrays that disagree with its sizes.
#pragma once

#include <new>
#include <stdexcept>

#include "host/matrix.hpp"
#include "tbsla_gb300.h"

#define TBSLA_API_CATCH                                       \
  catch (const std::bad_alloc&) { return TBSLA_ERR_ALLOC; }    \
  catch (const std::length_error&) { return TBSLA_ERR_ALLOC; } \
  catch (...) { return TBSLA_ERR_INVALID_ARG; }

namespace tbsla_impl {
inline void empty_after_failure(tbsla_matrix* m) {
  if (!m) return;
  m->invalidate();
  m->values.clear();
  m->idx0.clear();
  m->idx1.clear();
  m->info = tbsla_info{};
  m->info.NR = m->info.NC = 1;
}
}  // namespace tbsla_impl

#define TBSLA_API_CATCH_EMPTY(m)                                                                     \
  catch (const std::bad_alloc&) {                                                                    \
    tbsla_impl::empty_after_failure(m);                                                              \
    return TBSLA_ERR_ALLOC;                                                                          \
  }                                                                                                  \
  catch (const std::length_error&) {                                                                 \
    tbsla_impl::empty_after_failure(m);                                                              \
    return TBSLA_ERR_ALLOC;                                                                          \
  }                                                                                                  \
  catch (...) {                                                                                      \
    tbsla_impl::empty_after_failure(m);                                                              \
    return TBSLA_ERR_INVALID_ARG;                                                                    \
  }
