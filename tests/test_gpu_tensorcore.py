"""The FAST self-heating product on the tensor cores (tcgen05, BF16 view
factors times a hi+lo BF16 split of eps*sigma*T^4, FP32 accumulation in TMEM)
against a host evaluation of the same sum."""
import os

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

SIGMA = np.float32(5.67e-8)


def _bf16(x):
    """Round float32 to the nearest BF16 (ties to even), returned as float64."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def _host_q(prob, T, rounded, min_entries=None):
    """Q[s][f] = sum_g vf * eps sigma T[g][s]^4 (float64 accumulation).
    With ``rounded``, the operands the FAST product uses: BF16 V (+ residual
    in the tiles that carry one) times hi + lo BF16 W for the entries of
    tensor-core tiles, and FP32 V times FP32 W for the sparse remainder."""
    from binarytpm_gb300 import workloads

    es = np.float32(prob.emissivity) * SIGMA
    T2 = (T * T).astype(np.float32)
    W = (es * (T2 * T2)).astype(np.float32)          # [nf][ntau]
    vf = prob.dep_vf.astype(np.float64)
    rows = np.repeat(np.arange(prob.nf), np.diff(prob.dep_ptr))
    Wg = W[prob.dep_idx].astype(np.float64)
    if rounded:
        hi = _bf16(W)
        lo = _bf16((W - hi.astype(np.float32)).astype(np.float32))
        me = workloads.TC_MIN_ENTRIES if min_entries is None else min_entries
        _, inv, _, has_lo = workloads.tc_tile_structure(prob.nf, prob.dep_ptr, prob.dep_idx, prob.dep_vf, me)
        tile = inv >= 0
        vhi = _bf16(prob.dep_vf)
        vlo = _bf16((prob.dep_vf - vhi.astype(np.float32)).astype(np.float32))
        lo_of_entry = has_lo[np.maximum(inv, 0)] & tile if len(has_lo) else np.zeros(len(inv), bool)
        vt = vhi + np.where(lo_of_entry, vlo, 0.0)
        vf = np.where(tile, vt, vf)
        Wg = np.where(tile[:, None], (hi + lo)[prob.dep_idx], Wg)
    Q = np.zeros((prob.nf, T.shape[1]))
    np.add.at(Q, rows, vf[:, None] * Wg)
    return Q.T


@pytest.mark.parametrize("ntau,min_entries", [(48, 64), (300, 64), (720, 64), (720, 1), (720, 8192)])
def test_tensorcore_selfheating_matches_host(gpu_ctx, ntau, min_entries, monkeypatch):
    """The default split, every cell a tile (threshold 1), and every entry in
    the sparse remainder (threshold 8192: no cell of 128 x 64 can hold more)."""
    from binarytpm_gb300 import lib

    monkeypatch.setenv("ATPM_TC_MIN_ENTRIES", str(min_entries))
    prob, ref = golden("binary_s3s1")
    prob = prob.with_(ntau=ntau)
    rng = np.random.default_rng(ntau)
    s = lib.Solve(gpu_ctx, prob, precision=lib.FAST)
    shadow = (rng.random((prob.nf, ntau)) < 0.5).astype(np.int32)
    illum = (rng.random((prob.nf, ntau)) * 600).astype(np.float32)
    s.set_forcing(shadow, illum)
    s.set_thermal_inertia(200.0)
    s.initialise_temperatures()
    s.run()  # evolve so temperatures vary with facet and step
    T, _ = s.surface_temperature()
    q = s.selfheating_flux().astype(np.float64)
    q_bf = _host_q(prob, T, rounded=True, min_entries=min_entries)
    q_ex = _host_q(prob, T, rounded=False)
    scale = np.abs(q_bf).max()
    assert scale > 1.0
    assert np.max(np.abs(q - q_bf)) <= 1e-5 * scale, np.max(np.abs(q - q_bf)) / scale
    # compensated BF16 operands: close to the exact FP32 sum
    assert np.max(np.abs(q - q_ex)) <= 1e-3 * scale


def test_tensorcore_off_uses_gather(gpu_ctx, monkeypatch):
    from binarytpm_gb300 import lib

    prob, ref = golden("binary_s3s1")
    monkeypatch.setenv("ATPM_TC", "0")
    s = lib.Solve(gpu_ctx, prob, precision=lib.FAST)
    s.set_forcing(ref["shadow"], ref["illumination"])
    s.set_thermal_inertia(200.0)
    s.initialise_temperatures()
    T, _ = s.surface_temperature()
    q = s.selfheating_flux().astype(np.float64)
    q_ex = _host_q(prob, T, rounded=False)
    assert np.max(np.abs(q - q_ex)) <= 1e-5 * np.abs(q_ex).max()
