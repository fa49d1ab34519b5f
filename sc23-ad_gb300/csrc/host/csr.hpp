// Host-side sparse containers shared by the setup, the scheduler and the C ABI.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace sagb {

// FP64 CSR with sorted column indices inside each row (the layout of the
// reference's CSRMat, matrix/csrmat.hpp:13-22).
struct CsrD {
    int n = 0, m = 0;
    std::vector<int> rptr, cind;
    std::vector<double> val;
    int64_t nnz() const { return rptr.empty() ? 0 : rptr[n]; }
};

// Fixed-point CSR: int32 values with `bit` fractional bits (and `dbit` for the
// diagonal entries of triangular factors).
struct CsrI {
    int n = 0, m = 0;
    std::vector<int> rptr, cind;
    std::vector<int32_t> val;
    int bit = 0, dbit = 0;
    int64_t nnz() const { return rptr.empty() ? 0 : rptr[n]; }
};

template <typename T>
struct CsrT {
    int n = 0, m = 0;
    std::vector<int> rptr, cind;
    std::vector<T> val;
    int64_t nnz() const { return rptr.empty() ? 0 : rptr[n]; }
};

struct SetupError {
    std::string msg;
};

}  // namespace sagb
