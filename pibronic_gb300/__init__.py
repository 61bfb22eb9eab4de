"""GB300-native PIMC block evaluation for vibronic models (drop-in for Pibronic's ``pibronic.pimc``).

Modules: ``pimc`` (the engine API), ``stats`` / ``jackknife`` (estimators), ``vibronic_io`` (model
files), ``file_structure`` (data-set layout), ``plan`` (host precompute + device tables),
``synthetic`` (seeded models), ``build`` (nvcc build of the CUDA library).
"""
__version__ = "0.1.0"
