"""GB300-native ray-query path of rendiation: BVH traversal + wavefront executor.

The compute path is librdn.so (CUDA for sm_103a behind the C ABI in include/rdn.h);
this package holds its host-side mirror of the reference's interfaces (the
acceleration-structure system and trace calls in `raytracing`, the device task
graph and ray-traced AO in `task_graph`, the path tracer in `path_tracing`,
multi-GPU partitioning in `partition`) and the seeded workload generators.
"""

from . import native, scenes  # noqa: F401
from .raytracing import (  # noqa: F401
    AccelerationStructureSystem,
    BottomLevelAccelerationStructureBuildSource,
    TopLevelAccelerationStructureSourceInstance,
)
