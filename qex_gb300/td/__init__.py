"""3D Kohn-Sham numint SCF on GB300 (numint, generalized eigh, DIIS, density matrix)."""
