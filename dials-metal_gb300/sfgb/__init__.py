"""GB300-native spot finder: the dispersion-extended threshold and 3-D
spot labelling of dials-metal's src/spots/, as sm_103a CUDA kernels behind a
C ABI (include/sf_api.h). This package is the Python host side over that ABI.
"""
