"""GB300-native (sm_103a) GPU BVH pipeline of BVHTest: LBVH build, parallel Bittner13 optimizer and
closest-hit tracer behind the C ABI of include/bvhgb.h (libbvhgb.so)."""
from .native import BvhgbError, HIT_DTYPE, NODE_DTYPE, PIXEL_DTYPE, load  # noqa: F401

__all__ = ["BvhgbError", "HIT_DTYPE", "NODE_DTYPE", "PIXEL_DTYPE", "load"]
