// Minimal logger with the call shapes util/utilityFunctions.h uses; prints nothing.
#ifndef HLB_REFSHIM_LOG_LOGGER_H
#define HLB_REFSHIM_LOG_LOGGER_H
namespace hemelb::log {
struct Critical {}; struct Error {}; struct Warning {}; struct Info {}; struct Debug {}; struct Trace {};
struct Singleton {}; struct OnePerCore {};
struct Logger {
  template <class L> static bool ShouldDisplay() { return false; }
  template <class L, class S, class... A> static void Log(A&&...) {}
};
}  // namespace hemelb::log
#endif
