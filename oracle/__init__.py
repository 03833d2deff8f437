"""CPU oracle of the GPU BVH pipeline: test infrastructure only (see oracle.h)."""
