"""GB300-native LBVH build and closest-hit traversal (drop-in for the
tay10r/lbvh build + trace path).

The compute path is the CUDA library liblbvh_gb300.so (C ABI in
include/lbvh_gb300.h); this package is its Python host interface.
"""
from .api import (  # noqa: F401
    BOXES,
    Batch,
    BVH,
    HIT_DTYPE,
    LEAF_BIT,
    MISS,
    NODE_DTYPE,
    SPHERE_HIT_DTYPE,
    TRIANGLES,
    Builder,
    Context,
    LbvhError,
    SphereTraverser,
    Traverser,
    default_context,
    hits_view,
    make_triangles,
    sphere_boxes,
)
