"""GB300-native phonon hot path for PARPHOM: D(q) assembly, the pzheevx-
equivalent Hermitian eigensolve and group velocities behind a C ABI
(libparphom_gpu.so), with readers/writers for the reference's file formats."""
__version__ = "0.1.0"
