"""chromo_gb300: chromo's Monte Carlo inner loop on GB300 (sm_103a).

The public API mirrors the reference's (``polymers.Chromatin`` / ``SSWLC``,
``binders``, ``fields.UniformDensityField``, the ``mc`` move and controller
classes and ``mc.mc_sim``); the work runs in hand-written CUDA behind the C
ABI of ``include/chromo_gb300.h``.
"""
__version__ = "0.1.0"
