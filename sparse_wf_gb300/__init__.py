"""GB300-native FiRE local-energy hot path.

Hand-written sm_103a CUDA kernels behind a C ABI (``include/fire.h``, ``libfire.so``) for the
sparse forward-Laplacian local energy of the FiRE ``new_sparse`` wavefunction and its all-electron
Metropolis step; ``FireWaveFunction`` mirrors the reference's wavefunction interface.
"""
from .params import ModelDims, activate_jastrow, init_params, pack_params, param_offsets  # noqa: F401
from .systems import Molecule, alkane, hydrogen_chain, init_electrons, spin_counts  # noqa: F401


def __getattr__(name):
    # torch-dependent parts are imported lazily so that host-only tooling works without CUDA
    if name in ("FireWaveFunction", "StaticArgs", "DeviceParams", "make_local_energy", "make_mcmc"):
        from . import wavefunction

        return getattr(wavefunction, name)
    raise AttributeError(name)
