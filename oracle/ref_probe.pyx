# Test-only harness: exposes the reference's own `cdef` helpers that the
# sparse-PCA path uses but that brisc does not export to Python, so that the
# oracle restatement (oracle/oracle.c) can be pinned against them bit for bit.
# Built only by oracle/build_ref.py into oracle/_ref/; never shipped.
#
# Reference functions called (brisc/cyutils.pyx):
#   srand          :1228-1232   PCG32 seeding
#   random_normal  :1180-1191   Box-Muller in float
#   norm           :1089-1094   serial float32 2-norm
# and the start-vector recipe of brisc/pca.pyx:801-806.

import numpy as np
from brisc.cyutils cimport srand, random_normal, norm, rand


def start_vector(unsigned long long seed, unsigned num_genes):
    """V[:, 0] exactly as brisc/pca.pyx:683,801-806 builds it."""
    cdef unsigned long long state = srand(seed)
    cdef unsigned i
    cdef float inverse_norm
    out = np.empty(num_genes, dtype=np.float32)
    cdef float[::1] v = out
    for i in range(num_genes):
        v[i] = random_normal(&state)
    inverse_norm = 1 / norm(v)
    for i in range(num_genes):
        v[i] *= inverse_norm
    return out


def raw_normals(unsigned long long seed, unsigned count):
    """`count` successive random_normal draws after srand(seed)."""
    cdef unsigned long long state = srand(seed)
    cdef unsigned i
    out = np.empty(count, dtype=np.float32)
    cdef float[::1] v = out
    for i in range(count):
        v[i] = random_normal(&state)
    return out


def raw_rand(unsigned long long seed, unsigned count):
    """`count` successive PCG32 outputs after srand(seed)."""
    cdef unsigned long long state = srand(seed)
    cdef unsigned i
    out = np.empty(count, dtype=np.uint32)
    cdef unsigned[::1] v = out
    for i in range(count):
        v[i] = rand(&state)
    return out
