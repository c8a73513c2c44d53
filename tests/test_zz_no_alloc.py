"""fire_triplets_static -- the variant of fire_triplets that takes no workspace and allocates nothing --
against fire_triplets, both called through the C ABI.

The file name sorts last so that the GPU suite runs it after every other test, when the library's
kernels have already run many times; it must also pass on its own.  Each case makes two calls in a row
on different electron positions, so stale scratch from the first call would show up in the second.
Outputs are integer indices: the tolerance is bit-exact."""
import ctypes as C

import numpy as np
import pytest

from helpers import case, golden
from sparse_wf_gb300 import _lib


def _problem(g, mol, nu, B, cap_pairs, precision):
    return _lib.Problem(mol.n_el, nu, len(mol.Z), B, float(g["cutoff"]), float(g["cutoff_1el"]), cap_pairs, 1,
                        _lib.PREC[precision], 0)


def _call_both(lib, prob, r, cap, torch):
    """(outputs of fire_triplets, status) and (outputs of fire_triplets_static, status), [B, 4, cap]."""
    B = r.shape[0]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rt = torch.from_numpy(r).cuda()
    res = []
    for static in (False, True):
        outs = [torch.full((B, cap), -7, dtype=torch.int32, device="cuda") for _ in range(4)]
        status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device="cuda")
        ptrs = [C.c_void_p(o.data_ptr()) for o in outs]
        if static:
            rc = lib.fire_triplets_static(stream, C.byref(prob), C.c_void_p(rt.data_ptr()), cap, *ptrs,
                                          C.c_void_p(status.data_ptr()))
        else:
            ws = torch.empty(64 << 20, dtype=torch.uint8, device="cuda")
            rc = lib.fire_triplets(stream, C.byref(prob), C.c_void_p(rt.data_ptr()), cap, *ptrs,
                                   C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()), C.c_void_p(status.data_ptr()))
        assert rc == _lib.FIRE_OK
        torch.cuda.synchronize()
        res.append((np.stack([o.cpu().numpy() for o in outs], axis=1), status.cpu().numpy()))
    return res


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("name", ["h10", "c2h6"])
def test_static_scratch_matches_workspace_entry(cuda_lib, name, precision):
    import torch

    g = golden(name)
    mol, nu, r, *_ = case(name)
    B, cap = r.shape[0], g["triplets"].shape[2]
    cap_pairs = int(g["counts"][:, 0].max() + g["counts"][:, 1].max()) + 4
    dt = np.float64 if precision == "fp64" else np.float32
    # second call: moved electrons (other neighbour lists), larger triplet capacity
    r2 = (r + np.random.default_rng(7).normal(0.0, 0.4, r.shape)).astype(np.float32)
    for k, (rr, cp, ct) in enumerate(((r, cap_pairs, cap), (r2, 2 * cap_pairs, 2 * cap))):
        prob = _problem(g, mol, nu, B, cp, precision)
        (ref, st_ref), (got, st_got) = _call_both(cuda_lib, prob, np.ascontiguousarray(rr.astype(dt)), ct, torch)
        np.testing.assert_array_equal(got, ref, err_msg=f"call {k + 1}")
        np.testing.assert_array_equal(st_got[0], st_ref[0])
        assert st_got[0] == 0
        if k == 0:
            np.testing.assert_array_equal(got, g["triplets"])


@pytest.mark.gpu
def test_static_scratch_rejects_oversize(cuda_lib):
    _rejects_oversize(cuda_lib)


def test_static_scratch_rejects_oversize_on_host():
    """The size check runs before any CUDA call, so it is host logic (no pointer is dereferenced)."""
    _rejects_oversize(_lib.load())


def _rejects_oversize(lib):
    g = golden("c2h6")
    mol, nu, r, *_ = case("c2h6")
    n = mol.n_el
    cap_pairs = 64
    per_walker = 2 * n + 1 + 2 * cap_pairs  # deg, rowptr, nbr, rev
    fits = _lib.TRIPLETS_STATIC_MAX_WORDS // per_walker
    dummy = [C.c_void_p(256)] * 5
    for B, want in ((fits + 1, 2), (1 << 20, 2)):  # FIRE_ERR_UNSUPPORTED
        prob = _problem(g, mol, nu, B, cap_pairs, "fp32")
        rc = lib.fire_triplets_static(None, C.byref(prob), dummy[0], 128, *dummy[1:], C.c_void_p(512))
        assert rc == want
    prob = _problem(g, mol, nu, 4, cap_pairs, "fp32")
    assert lib.fire_triplets_static(None, C.byref(prob), None, 128, *dummy[1:], C.c_void_p(512)) == 1
