"""GB300-native (sm_103a) Capon/MVDR per-pixel path.

The compute is the CUDA library ``libcos_capon.so`` (C ABI in
``include/cos_capon.h``); ``cos_gb300.capon`` mirrors the reference's Capon
interface on top of it.  Importing the package does not load the library;
importing ``cos_gb300.capon`` does, and raises if it is missing.
"""
__all__ = ["capon", "synth", "build"]
