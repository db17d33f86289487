"""GB300-native forward/inverse harmonic transforms on SO(3) and S^2.

A drop-in for the transform path of fdcl-gwu/FFTSO3: the classes keep the
reference's names (FFTSO3_complex, FFTSO3_real, FFTS2_complex, FFTS2_real and
the FFTSO3_matrix / FFTS2_matrix containers) and call the CUDA library
libfftso3_gb300.so through its C ABI (include/fftso3_gb300.h).
"""
from .matrix import (FFTS2_matrix_complex, FFTS2_matrix_real, FFTSO3_matrix_complex, FFTSO3_matrix_real,
                     s2_index, s2_ncoeff, so3_index, so3_ncoeff, so3_offset)
from .rotation import R_to_euler323, euler323_to_R, expm_SO3, hat
from .transforms import FFTS2_complex, FFTS2_real, FFTSO3_complex, FFTSO3_real, alpha_j, beta_k, correlate_s2
from ._lib import Batch, FFTSO3Error, Plan
from .clebsch_gordan import Clebsch_Gordon_complex, Clebsch_Gordon_real

__all__ = [
    "FFTSO3_complex", "FFTSO3_real", "FFTS2_complex", "FFTS2_real",
    "FFTSO3_matrix_complex", "FFTSO3_matrix_real", "FFTS2_matrix_complex", "FFTS2_matrix_real",
    "so3_index", "so3_ncoeff", "so3_offset", "s2_index", "s2_ncoeff",
    "R_to_euler323", "euler323_to_R", "expm_SO3", "hat", "alpha_j", "beta_k", "correlate_s2", "FFTSO3Error", "Plan", "Batch", "Clebsch_Gordon_complex", "Clebsch_Gordon_real",
]
