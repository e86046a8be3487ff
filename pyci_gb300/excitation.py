r"""Excitation-level determinant sets (pyci/excitation_ci.py:23-39)."""

__all__ = ["add_excitations"]


def add_excitations(wfn, *excitations, ref=None):
    r"""Add the determinants of each excitation level in ``excitations`` to ``wfn``.

    Levels are taken relative to ``ref`` (default: the Hartree-Fock
    determinant), in the order given, with the wave function's own insertion
    order (``add_excited_dets``).
    """
    for e in excitations:
        wfn.add_excited_dets(e, ref=ref)
