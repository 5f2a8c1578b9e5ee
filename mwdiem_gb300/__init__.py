"""mwdiem_gb300 -- GB300 (sm_103a) implementation of MWDiEM's per-step DEM hot path.

Modules named like the reference's own (``gpu_fine_contact_detection``, ``gpu_Verlet``,
``LIBRARY_Coarse_contact_detection``, ``LIBRARY_Force``, ``Particle_class``) keep its call surface;
``sim`` is the device-resident, batched, graph-captured step; ``shapes`` and ``scene`` build inputs.
The compute path is ``libmwdem.so`` (hand-written CUDA, C ABI in ``include/mwdem.h``).
"""
__all__ = ["gpu_fine_contact_detection", "gpu_Verlet", "LIBRARY_Coarse_contact_detection", "shapes"]
__version__ = "0.1.0"
