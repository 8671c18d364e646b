"""The tensor-core dense commutator (obe_dense_commutator_tf32: tcgen05.mma kind::tf32, FP32
accumulators in tensor memory) against the commutator -i[H, rho] in complex128 on the host, for
random Hermitian H and rho at 16, 39 and 76 states.  TF32 keeps 10 mantissa bits of each operand,
so the tolerance is 4e-3 of the largest element (measured products of 76-term sums)."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from centrex_tlf_gb300 import _abi

pytestmark = pytest.mark.gpu


def _hermitian(rng, count, n):
    m = rng.normal(size=(count, n, n)) + 1j * rng.normal(size=(count, n, n))
    return m + m.conj().transpose(0, 2, 1)


@pytest.mark.parametrize("n", [16, 39, 76])
def test_dense_commutator_matches_host(n):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n)
    count = 200  # more states than SMs: the CTAs loop
    h = _hermitian(rng, count, n)
    r = _hermitian(rng, count, n) / n
    ref = -1j * (h @ r - r @ h)
    dev = torch.device("cuda:0")
    d_h = torch.tensor(h, dtype=torch.complex64, device=dev)
    d_r = torch.tensor(r, dtype=torch.complex64, device=dev)
    d_o = torch.full((count, n, n), float("nan"), dtype=torch.complex64, device=dev)
    d_s = torch.zeros(1, dtype=torch.int32, device=dev)
    lib = _abi.load_library()
    for _ in range(2):
        st = lib.obe_dense_commutator_tf32(count, n, d_h.data_ptr(), d_r.data_ptr(), d_o.data_ptr(), d_s.data_ptr(),
                                           ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
        assert st == _abi.OBE_OK
        torch.cuda.synchronize()
        assert int(d_s.item()) == 0
        got = d_o.cpu().numpy().astype(np.complex128)
        err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert err <= 4e-3, f"max error {err:.2e} of the largest element"


def test_dense_commutator_rejects_sizes_beyond_80():
    lib = _abi.load_library()
    assert lib.obe_dense_commutator_tf32(1, 81, 1, 1, 1, 1, None) == _abi.OBE_ERR_INVALID
