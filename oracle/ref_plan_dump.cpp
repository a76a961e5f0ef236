// ORACLE — test infrastructure only (never linked into the product).
//
// Driver that instantiates the reference's own host plan,
// bytecrt::make_rns_plan (native-smoke/rns-plan.hpp:174-324), for a
// q = 2^W - gap modulus and prints the plan as JSON, so that the oracle's
// restated plan can be pinned to the reference's compiled code.  The header
// is included from the reference checkout (see oracle/build_ref.sh); it is not
// copied here.
#include "rns-plan.hpp"

#include <cstdio>
#include <cstdlib>
#include <vector>

static void print_u32(const char* name, const std::vector<uint32_t>& v, bool comma = true) {
    std::printf("\"%s\": [", name);
    for (size_t i = 0; i < v.size(); ++i) std::printf(i ? ",%u" : "%u", v[i]);
    std::printf("]%s\n", comma ? "," : "");
}

int main(int argc, char** argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: ref_plan_dump N W gap\n");
        return 2;
    }
    const unsigned N = unsigned(std::strtoul(argv[1], nullptr, 10));
    const unsigned W = unsigned(std::strtoul(argv[2], nullptr, 10));
    const uint32_t gap = uint32_t(std::strtoul(argv[3], nullptr, 10));
    const unsigned L = (W + 31) / 32;
    std::vector<uint32_t> q(L, 0xFFFFFFFFu);
    q[0] = uint32_t(0) - gap;
    q[L - 1] = (uint32_t(1) << (W - 32 * (L - 1))) - 1;
    const bytecrt::RnsPlan plan = bytecrt::make_rns_plan(N, W, q);
    std::printf("{\"N\": %u, \"W\": %u, \"L\": %u, \"gap\": %u, \"P\": %u, \"kpad\": %u,\n",
                N, W, L, gap, plan.pcount, plan.kpad);
    print_u32("q", q);
    print_u32("primes", plan.primes);
    print_u32("psi", plan.psi_roots);
    print_u32("n_inverse", plan.n_inverse);
    print_u32("crt_inverse", plan.crt_inverse);
    // B4: 4L columns of kpad bytes each, column-major (rns-plan.hpp:301-322).
    std::vector<uint32_t> b4(plan.b_byte_matrix.begin(), plan.b_byte_matrix.end());
    print_u32("b4", b4, false);
    std::printf("}\n");
    return 0;
}
