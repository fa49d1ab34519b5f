// Matrix features for the learned fractional-bit selector.
//
// The reference chooses F_G from one number, c_max/||b|| of an FP64 V-cycle on
// b (Work/main.cpp:153-161).  The selector sees that number and the quantities
// that decide how much room the integer arithmetic has: the sizes and fill of
// the hierarchy, diagonal dominance and asymmetry of the fine operator, and the
// fractional bits each integer operator got from its own conversion rule.
#pragma once
#include "amg_setup.hpp"
#include "csr.hpp"

namespace sagb {

constexpr int kNumFeatures = 20;

// A: the scaled fine matrix; h: its integer hierarchy; ratio = c_max/||b||.
void bit_features(const CsrD &A, const IntHierarchy &h, double ratio, float *out);

}  // namespace sagb
