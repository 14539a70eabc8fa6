"""plainmp_gb300: GB300-native collision-checking hot path of plainmp.

Batched forward kinematics, sphere-vs-SDF checks (box, sphere, cylinder, ground, point
cloud), self-collision sphere pairs, motion-validator edge checks and constraint Jacobians,
as hand-written sm_103a CUDA kernels behind the C ABI in include/pmgpu.h.  The Python
modules mirror the reference's ``plainmp.kinematics``, ``plainmp.psdf``, ``plainmp.constraint``
and ``plainmp.kdtree`` interfaces.
"""
from ._lib import CudaError, DeviceTimeout, device_count  # noqa: F401
from .constraint import (ConstraintBase, EqCompositeCst, EqConstraintBase, IneqCompositeCst,  # noqa: F401
                         IneqConstraintBase, LinkPoseCst, LinkPositionBoundCst, SequentialCst, SphereAttachmentSpec,
                         SphereCollisionCst)
from .kdtree import KDTree  # noqa: F401
from .kinematics import BaseType, KinematicModel  # noqa: F401
from .motion_validator import BoxMotionValidator, EuclideanMotionValidator  # noqa: F401
from .psdf import (BoxSDF, ClosedPrimitiveSDFBase, CloudSDF, CylinderSDF, GroundSDF, Pose,  # noqa: F401
                   PrimitiveSDFBase, SDFBase, SphereSDF, UnionSDF)

__version__ = "0.1.0"
