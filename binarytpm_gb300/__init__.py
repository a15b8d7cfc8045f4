"""GB300-native BinaryTPM thermophysical hot path (package root).

The CUDA library (``libatpm``) is loaded by :mod:`binarytpm_gb300.lib`;
everything else here is host-side plumbing (synthetic meshes, reference file
formats, solve descriptions).
"""
