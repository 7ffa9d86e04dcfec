"""del_msh_gb300 — GB300-native (sm_103a) LBVH build and BVH ray cast with
del-msh's array layouts and call signatures.

Sub-packages mirror ``del_msh_dlpack``'s torch front-ends for this path:
``Mortons.torch``, ``Array1D.torch``, ``TriMesh3.torch``, ``Pix2Tri.torch``,
plus ``SearchBvh3.torch`` (del-msh-cpu ``search_bvh3::first_intersection_ray``
over ray arrays).  All of them run the CUDA library ``libdelmsh_gb300.so``;
CPU tensors are rejected (there is no CPU fallback).
"""
from ._native import DelMshError, device_status, load  # noqa: F401

__version__ = "0.1.0"
