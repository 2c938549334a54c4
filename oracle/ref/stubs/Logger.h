// Minimal logger for compiling GUNDAM's Cache::Manager calculators and its
// likelihood classes on the host outside the GUNDAM build (test
// infrastructure): informational output goes nowhere, errors throw
// std::runtime_error with the streamed message.
#ifndef GW_REF_STUB_LOGGER_H
#define GW_REF_STUB_LOGGER_H
#include <iostream>
#include <sstream>
#include <stdexcept>

namespace gw_ref_stub {
struct NullStream : std::ostream {
  NullStream() : std::ostream(nullptr) {}
};
inline NullStream& null_stream() {
  static NullStream s;
  return s;
}
}  // namespace gw_ref_stub

#define LogInfo gw_ref_stub::null_stream()
#define LogDebug gw_ref_stub::null_stream()
#define LogWarning gw_ref_stub::null_stream()
#define LogError gw_ref_stub::null_stream()
#define LogAlert gw_ref_stub::null_stream()
#define LogTrace gw_ref_stub::null_stream()
#define LogErrorOnce gw_ref_stub::null_stream()
#define LogErrorIf(cond_) gw_ref_stub::null_stream()
#define LogTraceIf(cond_) gw_ref_stub::null_stream()
#define LogScopeIndent \
  do {                 \
  } while (0)
#define GET_VAR_NAME_VALUE(var_) #var_ << " = " << (var_)
#define LogThrow(msg_)                   \
  do {                                   \
    std::ostringstream gw_ref_os_;       \
    gw_ref_os_ << msg_;                  \
    throw std::runtime_error(gw_ref_os_.str()); \
  } while (0)
#define LogThrowIf(cond_, msg_) \
  do {                          \
    if (cond_) LogThrow(msg_);  \
  } while (0)
#define LogExit(msg_) LogThrow(msg_)
#endif
