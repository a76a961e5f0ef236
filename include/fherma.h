// fherma.h — the C++ plugin ABI this library plugs into.
//
// The types must be layout-identical to the challenge's generated header
// (polymul/negacyclic@1.0.0, native-smoke/fherma.h:13-48) so that a generated
// main.cpp compiled against that header links against libfherma_gb300.so.
// With FHERMA_BATCHED defined, Point gains the leading batch size B and the
// tensors are [B][N][L] (polymul/negacyclic-batched@1.0.0,
// native-batched/fherma.h:27-49); build libfherma_gb300_batched.so for it.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace fherma {

template <class T>
struct Tensor {
    std::vector<int64_t> shape;
    std::vector<T> data;            // row-major

    int64_t count() const {
        int64_t n = 1;
        for (int64_t d : shape) n *= d;
        return n;
    }
};

struct Point {
#ifdef FHERMA_BATCHED
    uint32_t B = 0;                 // products per call
#endif
    uint32_t N = 0;                 // coefficients (power of two)
    uint32_t W = 0;                 // bits of q
    uint32_t L = 0;                 // uint32 limbs per coefficient
    Tensor<uint32_t> q;             // [L]
};

struct Inputs {
    Tensor<uint32_t> a;             // [N][L] (batched: [B][N][L])
    Tensor<uint32_t> b;
};

struct Outputs {
    Tensor<uint32_t> c;             // [N][L] (batched: [B][N][L])
};

}  // namespace fherma

void* fherma_init(const fherma::Point& p);
fherma::Outputs fherma_run(void* state, const fherma::Inputs& in);
void fherma_free(void* state);
