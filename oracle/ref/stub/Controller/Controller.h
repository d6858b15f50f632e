// Minimal stand-in for the reference's Controller/Controller.h so the
// reference's ExtendedOctree converter compiles outside the full library.
// TEST INFRASTRUCTURE ONLY (oracle/_ref).  Logging goes to a silent sink and
// performance counters are ignored.
#ifndef TVK_REF_STUB_CONTROLLER_H
#define TVK_REF_STUB_CONTROLLER_H

#include "Basics/PerfCounter.h"
#include "DebugOut/AbstrDebugOut.h"

namespace tuvok {

class QuietOut : public AbstrDebugOut {
 public:
  void printf(enum DebugChannel, const char*, const char*) override {}
  void printf(const char*) const override {}
};

class Controller {
 public:
  static Controller& Instance() {
    static Controller c;
    return c;
  }
  static const Controller& ConstInstance() { return Instance(); }
  AbstrDebugOut* DebugOut() { return &out_; }
  const AbstrDebugOut* DebugOut() const { return &out_; }
  void IncrementPerfCounter(enum PerfCounter, double) {}

 private:
  QuietOut out_;
};

}  // namespace tuvok

#define T_ERROR(...) do { tuvok::Controller::Instance().DebugOut()->Error(_func_, __VA_ARGS__); } while (0)
#define WARNING(...) do { tuvok::Controller::Instance().DebugOut()->Warning(_func_, __VA_ARGS__); } while (0)
#define MESSAGE(...) do { tuvok::Controller::Instance().DebugOut()->Message(_func_, __VA_ARGS__); } while (0)
#define OTHER(...) do { tuvok::Controller::Instance().DebugOut()->Other(_func_, __VA_ARGS__); } while (0)

#endif
