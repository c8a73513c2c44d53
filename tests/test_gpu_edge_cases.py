"""Edge cases of the local-energy path through the C ABI: an electron with an empty e-e neighbour list (its row of the
sparse Jacobian holds only the self position, its pair lists and triplets are empty)."""
import numpy as np
import pytest

from sparse_wf_gb300 import systems
from sparse_wf_gb300.wavefunction import FireWaveFunction

from test_gpu_parity import _check_local_energy

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp32", "fp64", "mixed"])
def test_local_energy_isolated_electron(cuda_lib, precision):
    """H4 chain plus a hydrogen 30 bohr away whose electron sits near its nucleus: that electron has no e-e
    neighbours; E_loc, log|psi|, its gradient and Laplacian against the oracle with the parity tolerances."""
    from make_golden import make_params

    R = np.array([[0.0, 0, 0], [1.8, 0, 0], [3.6, 0, 0], [5.4, 0, 0], [35.4, 0, 0]], np.float32)
    mol = systems.Molecule("H4+H", R, np.ones(5, np.int64))
    nu, _ = systems.spin_counts(mol)
    rng = np.random.default_rng(2)
    r = np.stack([np.concatenate([R[:4] + 0.5 * rng.standard_normal((4, 3)),
                                  R[4:] + 0.3 * rng.standard_normal((1, 3))]) for _ in range(3)]).astype(np.float32)
    _, p, _, _ = make_params(mol, nu, r[0], seed=3, activate=True)
    wf = FireWaveFunction(mol, precision=precision)
    _check_local_energy(wf, mol, nu, r, p, precision)
