"""The jax.ffi custom calls (sparse_wf_gb300/jax_ffi.py over xla/fire_xla.cc) against the ctypes path: the same
library entry points on the same inputs, so the results must agree bit for bit.  Needs jax with CUDA and jaxlib's
FFI header; skipped where jax is not installed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_local_energy_custom_call_matches_ctypes(cuda_lib):
    jax = pytest.importorskip("jax")
    import jax.numpy as jnp
    import torch

    from helpers import case
    from sparse_wf_gb300 import build, jax_ffi
    from sparse_wf_gb300.wavefunction import FireWaveFunction, StaticArgs

    if build.build_xla() is None:
        pytest.skip("jaxlib ships no FFI header here")
    jax.config.update("jax_enable_x64", True)
    mol, nu, r, p, _, _ = case("c2h6")
    wf = FireWaveFunction(mol, precision="mixed")
    wf.refine = False  # the custom call runs without the refinement pass
    dp = wf._params(p)
    rr = torch.from_numpy(r).cuda()
    s = wf.get_static_input(rr)
    static = StaticArgs(s.n_pairs_same, s.n_pairs_diff, s.n_triplets, s.n_neighbours_en)
    e_ref, aux = wf.local_energy_full(dp, rr, static)
    e, logpsi, sign, stats, status = jax_ffi.local_energy(
        jnp.asarray(dp.prepared.cpu().numpy()), jnp.asarray(wf.R), jnp.asarray(wf.Z.astype(np.float32)),
        jnp.asarray(r), static, nu, precision=1)
    assert int(np.asarray(status)[0]) == 0
    np.testing.assert_array_equal(np.asarray(e), e_ref.cpu().numpy())
    np.testing.assert_array_equal(np.asarray(logpsi), aux["logpsi"].cpu().numpy())


def test_logpsi_grad_custom_call_matches_ctypes(cuda_lib):
    """The parameter-gradient custom call (FireLogpsiGrad) gives the rows of fire_logpsi_grad through ctypes."""
    jax = pytest.importorskip("jax")
    import jax.numpy as jnp
    import torch

    from helpers import case
    from sparse_wf_gb300 import build, jax_ffi
    from sparse_wf_gb300.wavefunction import FireWaveFunction, StaticArgs

    if build.build_xla() is None:
        pytest.skip("jaxlib ships no FFI header here")
    mol, nu, r, p, _, _ = case("c2h6")
    wf = FireWaveFunction(mol, precision="fp32")
    dp = wf._params(p)
    rr = torch.from_numpy(r).cuda()
    s = wf.get_static_input(rr)
    static = StaticArgs(s.n_pairs_same, s.n_pairs_diff, s.n_triplets, s.n_neighbours_en)
    g_ref, _, lp_ref = wf.logpsi_grad(dp, rr, static, chunk=len(r))
    g, logpsi, sign, status = jax_ffi.logpsi_grad(jnp.asarray(dp.prepared.cpu().numpy()), jnp.asarray(wf.R),
                                                  jnp.asarray(r), static, nu, int(g_ref.shape[1]), chunk=len(r))
    assert int(np.asarray(status)[0]) == 0
    np.testing.assert_array_equal(np.asarray(g), g_ref.cpu().numpy())
    np.testing.assert_array_equal(np.asarray(logpsi), lp_ref.cpu().numpy())
