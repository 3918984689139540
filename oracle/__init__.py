"""CPU oracle for the Kohn-Sham SCF hot path (test infrastructure only).

This package is a NumPy float64 restatement of the reference algorithm
(qedft ``qedft/train/od/*.py`` plus the jax_dft primitives it calls, and the
3D numint / generalized-eigh / DIIS / rdm1 pieces of ``qedft/train/td``).
It exists to check the CUDA path; it is never the thing measured or shipped.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
arm may import it.  The product package ``qex_gb300`` never imports it and has
no CPU fallback.

Parity pins (what ties this restatement to the reference):
  * E_xc known-answer value and the dx-scaled v_xc of
    ``tests/test_scf_od.py:38-86`` / ``tests/test_jit_scf_od.py:40-88``;
  * converged-flag sequences of ``tests/test_scf_od.py:184-215`` and
    ``tests/test_jit_scf_od.py:186-229``;
  * the shipped exponential-Coulomb chain potentials
    ``data/od/{h2,h2_h2,h4}/external_potentials.npy`` (to ~1e-15);
  * the shipped exact KS potentials ``data/od/h2/exact_v_s.npy`` whose
    non-interacting densities reproduce ``data/od/h2/densities.npy`` with the
    five-point kinetic stencil (to ~1.5e-5 L2);
  * ``tests/test_make_rdm1.py`` and ``tests/test_generalized_eigh_padded.py``
    semantics for the 3D pieces.
Parity unpinned: the exponential-Coulomb LDA constants (jax_dft ``xc.py`` is
not in the reference tree; restated from the published uniform-gas fit of
Baker et al., Phys. Rev. B 91, 235141 (2015)).
"""
