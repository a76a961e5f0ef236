"""The reference's own encode and CRT kernels on the same GPU.

encode_mma32 (native-smoke/rns-encode-mma.cuh:148-252) and g1_crt32
(native-smoke/g1-crt.cuh:201-335), compiled unmodified from the reference
checkout into oracle/_ref/ref_kernels.cubin, are launched as the reference's
launchers do; their outputs are checked against the oracle, and this library's
encode and CRT kernels must take less time per product at both geometries the
reference supports, one product per launch as the reference launches them.
"""
import numpy as np
import pytest

from conftest import package
from oracle import ref_kernels

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

GAP = 0x9E3779B1


def ours_us(N, W, q, group, reps=4):
    """Per-product stage times of this library (CUDA events around each stage)."""
    pkg = package()
    m = pkg.Multiplier(N, W, q)
    m.set_group(group)
    a = np.stack([pkg.inputs.uniform(q, N, 11 + i) for i in range(group)])
    b = np.stack([pkg.inputs.uniform(q, N, 51 + i) for i in range(group)])
    da = torch.from_numpy(a.view(np.int32)).cuda()
    db = torch.from_numpy(b.view(np.int32)).cuda()
    dc = torch.empty_like(da)
    st = torch.cuda.Stream()
    for _ in range(2):
        m.multiply_device(da, db, dc, group, stream=st.cuda_stream)
    m.synchronize()
    m.read_profile(reset=True)
    m.profile(True, every=1)
    for _ in range(reps):
        m.multiply_device(da, db, dc, group, stream=st.cuda_stream)
    m.synchronize()
    p = m.read_profile(reset=True)
    m.profile(False)
    return {k: 1000.0 * v / (reps * group) for k, v in p["ms"].items()}


@pytest.mark.skipif(not ref_kernels.available(),
                    reason="oracle/_ref/ref_kernels.cubin is built from the reference checkout by oracle/build_ref.sh")
@pytest.mark.parametrize("N,W", [(32768, 868), (65536, 1747)])
def test_reference_kernels_checked_and_slower(N, W):
    ref = ref_kernels.run(N, W, gap=GAP, reps=5)
    assert ref["checked"]
    ours = ours_us(N, W, ref_kernels.gap_modulus(W, GAP), group=1)
    assert ours["encode"] < ref["encode_mma32_us"], (ours, ref)
    assert ours["crt"] < ref["g1_crt32_us"], (ours, ref)
