// TEST INFRASTRUCTURE ONLY.  Stand-in for easylogging++, which the
// reference's include/spin/SpinInteraction.h includes: LOG(level) << ...
// compiles to a statement that never runs.
#pragma once
#include <iostream>
#define LOG(level) if (false) std::cerr
