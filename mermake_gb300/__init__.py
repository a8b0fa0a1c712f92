"""GB300 (sm_103a) implementation of MERMAKE's per-FOV image path.

The public names mirror ``mermake``'s modules: ``deconvolver.Deconvolver`` /
``full_deconv``, ``blur.box`` / ``box_2d`` / ``box_1d``, ``maxima.find_local_maxima``,
``fill.reflect``, ``math.subtract_clamp`` / ``subtract_reflect``,
``align.Aligner`` / ``DualAligner`` / ``drift`` / ``drift_save``.  Every
computation runs in ``libmermake_gb300.so`` (CUDA, sm_103a) through the C ABI
declared in ``include/mermake_gb300.h``; arrays are torch CUDA tensors.
"""
__version__ = "0.1.0"
REFERENCE_VERSION = "0.0.74"
