// ORACLE — test and measurement infrastructure only (never linked into the
// product).
//
// Instantiates the reference's own encode and CRT kernels, unmodified, so that
// they can be timed on the same GB300 as this library's kernels:
//   bytecrt::encode_mma32<L, P, Kpad, true>   native-smoke/rns-encode-mma.cuh:148-252
//   bytecrt::g1_crt32<W, L, P, Kpad, true>     native-smoke/g1-crt.cuh:201-335
// at the two geometries the reference supports (N=65536/W=1747 and
// N=32768/W=868).  The headers are included from the reference checkout (see
// oracle/build_ref.sh, which compiles this file to a device-only cubin in
// oracle/_ref/); nothing of the reference is copied here.  oracle/ref_kernels.py
// loads the cubin through the CUDA driver API and launches the kernels with the
// reference launchers' grids (rns-encode-mma.cuh:302-315, g1-crt.cuh:375-387).
#include "rns-encode-mma.cuh"
#include "g1-crt.cuh"

namespace bytecrt {
template __global__ void encode_mma32<55, 114, 224, true>(unsigned, const uint32_t*, const uint8_t*,
                                                          const uint32_t*, const uint64_t*, uint32_t*, unsigned);
template __global__ void encode_mma32<28, 57, 128, true>(unsigned, const uint32_t*, const uint8_t*,
                                                         const uint32_t*, const uint64_t*, uint32_t*, unsigned);
template __global__ void g1_crt32<1747, 55, 114, 480, true>(const uint8_t*, const uint8_t*, const float*,
                                                            const uint32_t*, uint32_t, uint32_t*, unsigned);
template __global__ void g1_crt32<868, 28, 57, 256, true>(const uint8_t*, const uint8_t*, const float*,
                                                          const uint32_t*, uint32_t, uint32_t*, unsigned);
}  // namespace bytecrt
