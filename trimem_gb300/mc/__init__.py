"""Device-resident drivers over the C ABI: the hybrid HMC + flip chain
(``device``), the effective-sample-size estimator (``ess``), energy
minimisation (``minim``) and trajectory / checkpoint output (``output``).

The reference's own Monte Carlo layer (``trimem.mc``) runs unchanged over
``trimem_gb300.core``: map ``sys.modules["trimem.core"]`` to it before
importing ``trimem.mc``.
"""
