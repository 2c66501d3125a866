"""GB300-native kD-tree Barnes-Hut N-body step.

The hot path of MarkCLewis/MultiLanguageKDTree (tree build, centre-of-mass pass,
theta-opening traversal, kick-drift) as hand-written sm_103a CUDA kernels behind a C ABI
(``include/kdnbody.h``, ``libkdnbody.so``).  This package is the Python host side: a
ctypes binding and the reference's module surface (``array_kd_tree``, ``array_particle``).
"""
from . import array_particle
from .quickstat import quickstat_index
from .array_kd_tree import (KDError, KDTreeSim, allocate_node_vec, build_tree, calc_accel,
                            fp32_peak, nodes_needed, simple_sim)
from .array_particle import PARTICLE_DTYPE, circular_orbits, plummer, ring, two_bodies

__all__ = ["KDTreeSim", "KDError", "allocate_node_vec", "nodes_needed", "build_tree",
           "calc_accel", "simple_sim", "PARTICLE_DTYPE", "circular_orbits", "ring", "plummer",
           "two_bodies", "array_particle", "quickstat_index", "fp32_peak"]
