"""Batched tridiagonal solves (the ADI line solve on arbitrary systems):
the generator and oracle on the CPU, the C-ABI kernels on the GPU."""
import numpy as np
import pytest

from geothermalwells_gb300 import _lib
from geothermalwells_gb300 import workloads as W
import oracle as O


def test_generator_properties():
    w = W.tridiagonal_batch(nsys=300, lmin=32, lmax=90, seed=3)
    a, b, c = w["a"], w["b"], w["c"]
    assert np.all(b >= 1.0 + np.abs(a) + np.abs(c) - 1e-12)        # diagonal dominance
    assert w["unknowns"] == int(w["slot_len"].sum())
    g0 = w["group_len"][0]
    rows = np.arange(g0)
    A = a[:32 * g0].reshape(g0, 32)
    assert np.all(A[0] == 0.0)
    lens = w["slot_len"][:32]
    pad = rows[:, None] >= lens[None, :]
    assert np.all(w["b"][:32 * g0].reshape(g0, 32)[pad] == 1.0)
    assert np.all(w["d"][:32 * g0].reshape(g0, 32)[pad] == 0.0)


def test_oracle_solves():
    w = W.tridiagonal_batch(nsys=500, lmin=32, lmax=200, seed=4)
    x = O.tridiag_batch(w)
    assert O.tridiag_residual(w, x) < 1e-14


def _gpu_solve(torch, w, precision):
    dev = {k: torch.from_numpy(np.ascontiguousarray(w[k])).cuda() for k in "abcd"}
    goff = torch.from_numpy(w["group_off"].astype(np.int64)).cuda()
    glen = torch.from_numpy(w["group_len"].astype(np.int32)).cuda()
    x = torch.zeros(w["n"], dtype=torch.float64, device="cuda")
    scratch = torch.zeros((w["n"] * 12 + 7) // 8, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    L = _lib.load()
    _lib.check(L.gw_tridiag_batch(precision, w["ngroups"], goff.data_ptr(), glen.data_ptr(),
                                  dev["a"].data_ptr(), dev["b"].data_ptr(), dev["c"].data_ptr(),
                                  dev["d"].data_ptr(), x.data_ptr(), scratch.data_ptr(), w["n"],
                                  torch.cuda.current_stream().cuda_stream))
    return x.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(_lib.GW_PREC_FP64, 1e-12), (_lib.GW_PREC_MIXED, 1e-10)])
def test_gpu_matches_oracle(precision, tol, gwlib, torch_cuda):
    w = W.tridiagonal_batch(nsys=3000, lmin=32, lmax=400, seed=6)
    ref = O.tridiag_batch(w)
    x = _gpu_solve(torch_cuda, w, precision)
    assert np.max(np.abs(x - ref)) / np.max(np.abs(ref)) < tol
    assert O.tridiag_residual(w, x) < (1e-14 if precision == _lib.GW_PREC_FP64 else 1e-12)


@pytest.mark.gpu
def test_gpu_edge_lengths(gwlib, torch_cuda):
    """Length-1 and length-2 systems and a batch that is not a multiple of 32."""
    w = W.tridiagonal_batch(nsys=45, lmin=1, lmax=3, seed=7)
    ref = O.tridiag_batch(w)
    for p in (_lib.GW_PREC_FP64, _lib.GW_PREC_MIXED):
        x = _gpu_solve(torch_cuda, w, p)
        assert np.max(np.abs(x - ref)) / np.max(np.abs(ref)) < 1e-10
