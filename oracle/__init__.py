"""CPU oracle for the MERMAKE per-FOV image path -- TEST INFRASTRUCTURE ONLY.

This package restates, on the CPU, what the reference (deprekate/MERMAKE
v0.0.74) computes on the per-FOV path, so that the GPU implementation in
``mermake_gb300`` can be checked against it.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import it, and only as the checker.  The product path never calls into it.

Modules
-------
deconv     FP64 NumPy/SciPy restatement of ``mermake/deconvolver.py``
           (Wiener spectrum, tile padding/reflect, FFT deconvolution, blur
           subtraction, stitching).
ckernels   ctypes wrapper around ``kernels.c``: a plain-C restatement of the
           reference kernels in ``mermake/maxima.cu`` (maxima count/collect,
           ``delta_fit_cross_corr``), ``mermake/blur.cu`` (``box_1d``) and
           ``mermake/fill.py`` (``mirror``).
align      NumPy/SciPy restatement of ``mermake/align.py`` and
           ``mermake/utils.py:fftconvolve``.
pipeline   restatement of the per-FOV call sequence of ``mermake/__main__.py``
           (DAPI block, hyb tile loop with keep-filter and offset).
synth      seeded synthetic stacks with the shapes of the benchmark
           configurations (Poisson background + Gaussian puncta, nuclei).

Parity of ``deconv`` is pinned by the reference's golden deconvolution slices
(``tests/examples/single/out/deconv.{300,500}.*.npz``, subsampled into
``tests/golden/``); ``ckernels`` is pinned by the reference's unit-test known
answers and, where ``oracle/_ref`` is built, by the reference kernels
themselves compiled as C++; ``align`` is pinned by the drift pickle shipped
with the reference.
"""
