"""GB300-native WaterGAP2 daily step: vertical water balance + lateral routing.

The compute path is the in-tree CUDA library ``_build/libwg_gpu.so`` (sm_103a),
reached through its C ABI (``include/wg_gpu.h``); ``watergap2_gb300.gpu`` binds
it.  ``region`` and ``synthetic`` describe and generate inputs and need no GPU.
"""
__all__ = ["region", "synthetic"]
