"""GB300-native ray-query engine for the Candela renderer's hot path.

SAH-BVH closest-hit / any-hit ray queries (stack and stackless traversal, reference buffer
formats) plus the diffuse-GI / RTAO ray generation and shading that consume them, as hand-written
sm_103a CUDA behind a C ABI (include/rq.h, candela_gb300/lib/librq.so).
"""
from . import scenes  # noqa: F401
from ._lib import (HIT_DTYPE, RAY_DTYPE, VERTEX_DTYPE, RqError)  # noqa: F401
from .engine import (BVH8Q, STACK, STACKLESS, BVH, Context, RayIntersector, Scene,  # noqa: F401
                     build_bvh, identity_entity, validate_scene)
