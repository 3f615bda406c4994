"""GB300-native (sm_103a) sweep-and-prune broadphase and particle
rigid-body step, behind the C ABI of include/gsap.h.

The compute path is libgsap.so (hand-written CUDA kernels under csrc/);
this package is the host-side mirror of the reference's ``Sap`` and
``ParticleRigidBody`` classes.  PyTorch is used only for device memory and
streams.
"""
from ._lib import (AXIS_PCA, AXIS_REF, CONTACT_CONFIG, CONTACT_REF, FLAG_GRAPH, FLAG_SORTED, FLAG_TEMPORAL,
                   MODE_AABB, MODE_SPHERE, GsapError, load)

__all__ = ["Sap", "ParticleRigidBody", "GsapError", "load", "MODE_AABB", "MODE_SPHERE", "AXIS_PCA",
           "AXIS_REF", "FLAG_SORTED", "FLAG_GRAPH", "FLAG_TEMPORAL", "CONTACT_REF", "CONTACT_CONFIG"]


def __getattr__(name):
    if name == "Sap":
        from .sap import Sap
        return Sap
    if name == "ParticleRigidBody":
        from .rigid import ParticleRigidBody
        return ParticleRigidBody
    raise AttributeError(name)
