"""atpm_scattering_noalloc: the scattering computation for callers that
cannot allocate device memory, with its scratch in a fixed device array.

It is checked against the allocating entry point (atpm_scattering on a solve
handle) through the C ABI: same inputs, bit-identical illumination, on two
calls in a row (the second call reuses the scratch the first one left
behind).  This file is collected last so a failure here does not hide the
other GPU tests.
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, dtype)).to(torch.device("cuda", 0))


def test_noalloc_scattering_matches_allocating_entry_point(gpu_ctx):
    torch = pytest.importorskip("torch")
    from binarytpm_gb300 import lib

    prob, _ = golden("binary_s3s1")
    s = lib.Solve(gpu_ctx, prob, precision=lib.REFERENCE)
    s.geometry_shadow()
    shadow, cosil = s.shadow(), s.cosillum()
    s.scattering()
    want = s.illumination()
    s.close()

    ptr = _dev(torch, prob.dep_ptr, np.int32)
    idx = _dev(torch, prob.dep_idx, np.int32)
    vf = _dev(torch, prob.dep_vf, np.float32)
    cs = _dev(torch, cosil, np.float32)
    sh = _dev(torch, shadow, np.uint8)
    status = torch.zeros(1, dtype=torch.int32, device="cuda:0")
    solar = float(np.float32(1367.0 / (prob.polar[0] * prob.polar[0])))
    L = lib.load()
    for _ in range(2):
        out = torch.full((prob.nf, prob.ntau), float("nan"), dtype=torch.float32, device="cuda:0")
        status.zero_()
        rc = L.atpm_scattering_noalloc(prob.nf, prob.ntau, ptr.data_ptr(), idx.data_ptr(), vf.data_ptr(),
                                       cs.data_ptr(), sh.data_ptr(), solar, prob.albedo,
                                       prob.scattering_accuracy, 1, out.data_ptr(), status.data_ptr(), None)
        assert rc == 0, L.atpm_last_error()
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        got = out.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu_ctx):
    torch = pytest.importorskip("torch")
    from binarytpm_gb300 import lib

    L = lib.load()
    buf = torch.zeros(16, dtype=torch.float32, device="cuda:0")
    p = buf.data_ptr()
    rc = L.atpm_scattering_noalloc(2048, 1024, p, p, p, p, p, 1367.0, 0.1, 1e-4, 1, p, p, None)
    assert rc == 4  # ATPM_E_UNSUPPORTED
    assert b"exceeds" in L.atpm_last_error()
