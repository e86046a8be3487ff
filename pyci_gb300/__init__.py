r"""pyci_gb300: PyCI's CI hot path on NVIDIA GB300 (sm_103a).

Drop-in for the ``pyci`` names on the sparse-operator path
(pyci/__init__.py:18-31): ``secondquant_op`` (alias ``hamiltonian``), the
``doci_wfn`` / ``fullci_wfn`` / ``genci_wfn`` wave functions, ``sparse_op``
(CSR build, ``op(x)``, ``op.solve``, ``op.update``), ``add_hci`` (heat-bath
CI selection), ``compute_rdms`` / ``compute_transition_rdms`` (with ``spinize_rdms`` and
``reduce_senzero_integrals``), ``compute_enpt2``, ``popcnt``, ``ctz``, thread-count helpers and
``add_excitations``.  The operator runs on the GPU through
``libpyci_gb300.so``; importing works without a GPU, building an operator
does not.

The native parts are built in-tree by ``python pyci_gb300/build.py`` (or
``__graft_entry__.build()``); importing fails loudly if they are missing.
"""

import os as _os

_HERE = _os.path.dirname(_os.path.abspath(__file__))

try:
    from pyci_gb300._pyci import (  # noqa: F401
        __version__,
        add_hci,
        compute_enpt2,
        compute_rdms,
        compute_transition_rdms,
        c_double,
        c_long,
        c_ulong,
        ctz,
        doci_wfn,
        fullci_wfn,
        genci_wfn,
        get_num_threads,
        gpu_version,
        one_spin_wfn,
        popcnt,
        secondquant_op,
        set_num_threads,
        sparse_op,
        two_spin_wfn,
        wavefunction,
    )
except ImportError as exc:  # pragma: no cover - exercised only on a broken build
    raise ImportError(
        "pyci_gb300's native module is not built; run `python pyci_gb300/build.py` "
        "(needs nvcc for sm_103a): " + str(exc)
    ) from exc

from pyci_gb300.excitation import add_excitations  # noqa: E402,F401
from pyci_gb300.utility import reduce_senzero_integrals, spinize_rdms  # noqa: E402,F401

hamiltonian = secondquant_op

LIBRARY_PATH = _os.path.join(_HERE, "lib", "libpyci_gb300.so")

__all__ = [
    "__version__",
    "c_long",
    "c_ulong",
    "c_double",
    "secondquant_op",
    "hamiltonian",
    "wavefunction",
    "one_spin_wfn",
    "two_spin_wfn",
    "doci_wfn",
    "fullci_wfn",
    "genci_wfn",
    "sparse_op",
    "get_num_threads",
    "set_num_threads",
    "popcnt",
    "ctz",
    "add_excitations",
    "add_hci",
    "compute_enpt2",
    "compute_rdms",
    "compute_transition_rdms",
    "reduce_senzero_integrals",
    "spinize_rdms",
    "gpu_version",
    "LIBRARY_PATH",
]
