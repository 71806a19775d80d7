"""GB300-native volumetric path tracer with a neural radiance cache (rtcamp8 hot path).

The compute path is the in-tree CUDA library librtc8_gb300.so (C ABI in include/); this
package holds its ctypes binding and the host-side mirror of the reference's renderer loop.
"""
__all__ = ["configs", "renderer"]
