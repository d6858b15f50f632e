// Minimal stand-in for the reference's Controller/StackTimer.h (timers are
// no-ops here).  TEST INFRASTRUCTURE ONLY (oracle/_ref).
#ifndef TVK_REF_STUB_STACK_TIMER_H
#define TVK_REF_STUB_STACK_TIMER_H

#include "Basics/PerfCounter.h"

namespace tuvok {
struct StackTimer {
  explicit StackTimer(enum PerfCounter) {}
};
}  // namespace tuvok

#define TimedStatement(pc, block) do { block; } while (0)

#endif
