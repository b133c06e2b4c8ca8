"""Rigid-body kinematics with forward-mode dual numbers.

Mirrors vlm/include/vlm_kinematics.hpp: a tree of nodes, each a function
t -> 4x4 homogeneous transform evaluated on a dual number (value and d/dt),
chained to its parent (transform_dual = parent(t) . own(t)).  The UVLM and
HBVLM drivers evaluate the transforms and their time derivatives on the host
for every step and hand them to the device, which applies them per vertex.

Matrices are 4x4 nested lists M[row][col] of Dual; ``to_colmajor`` flattens
them column-major like linalg::mat::store in the reference.
"""
import math

import numpy as np

__all__ = ["Dual", "sin", "cos", "translation_matrix", "rotation_matrix", "KinematicNode", "KinematicsTree",
           "Assembly", "matmul"]


class Dual:
    """a + b eps with eps^2 = 0 (headeronly/tinyad.hpp fwd::Number).  val and
    grad may be numpy arrays, so a whole time series evaluates at once."""
    __slots__ = ("val", "grad")

    def __init__(self, val, grad=0.0):
        self.val = val
        self.grad = grad

    @staticmethod
    def lift(x):
        return x if isinstance(x, Dual) else Dual(x, 0.0)

    def __add__(self, o):
        o = Dual.lift(o)
        return Dual(self.val + o.val, self.grad + o.grad)

    __radd__ = __add__

    def __sub__(self, o):
        o = Dual.lift(o)
        return Dual(self.val - o.val, self.grad - o.grad)

    def __rsub__(self, o):
        return Dual.lift(o) - self

    def __mul__(self, o):
        o = Dual.lift(o)
        return Dual(self.val * o.val, self.val * o.grad + self.grad * o.val)

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = Dual.lift(o)
        return Dual(self.val / o.val, (self.grad * o.val - self.val * o.grad) / (o.val * o.val))

    def __neg__(self):
        return Dual(-self.val, -self.grad)

    def __repr__(self):
        return "Dual(%r, %r)" % (self.val, self.grad)


def sin(x):
    x = Dual.lift(x)
    return Dual(np.sin(x.val), np.cos(x.val) * x.grad)


def cos(x):
    x = Dual.lift(x)
    return Dual(np.cos(x.val), -np.sin(x.val) * x.grad)


def _I():
    return [[Dual(1.0 if r == c else 0.0) for c in range(4)] for r in range(4)]


def matmul(a, b):
    return [[sum((a[r][k] * b[k][c] for k in range(4)), Dual(0.0)) for c in range(4)] for r in range(4)]


def translation_matrix(t):
    """vlm_kinematics.hpp translation_matrix: translation in the last column."""
    m = _I()
    for r in range(3):
        m[r][3] = Dual.lift(t[r])
    return m


def rotation_matrix(point, axis, angle):
    """Rodrigues rotation about `axis` through `point` (vlm_kinematics.hpp rotation_matrix)."""
    angle = Dual.lift(angle)
    ax = [float(a) for a in axis]
    # skew(a) as in the reference (columns {0,a.z,-a.y},{-a.z,0,a.x},{a.y,-a.x,0})
    K = [[0.0, -ax[2], ax[1]], [ax[2], 0.0, -ax[0]], [-ax[1], ax[0], 0.0]]
    K2 = [[sum(K[r][k] * K[k][c] for k in range(3)) for c in range(3)] for r in range(3)]
    s, c1 = sin(angle), Dual(1.0) - cos(angle)
    R = [[Dual(1.0 if r == c else 0.0) + s * K[r][c] + c1 * K2[r][c] for c in range(3)] for r in range(3)]
    p = [float(x) for x in point]
    m = _I()
    for r in range(3):
        for c in range(3):
            m[r][c] = R[r][c]
        m[r][3] = Dual(p[r]) - sum((R[r][k] * p[k] for k in range(3)), Dual(0.0))
    return m


class KinematicNode:
    def __init__(self, fn=None):
        self.fn = fn or (lambda t: _I())
        self.parent = None

    def after(self, parent):
        self.parent = parent
        return self

    def transform_dual(self, t):
        own = self.fn(Dual(float(t), 1.0))
        return matmul(self.parent.transform_dual(t), own) if self.parent else own

    def transform(self, t):
        m = self.transform_dual(t)
        return np.array([[m[r][c].val for c in range(4)] for r in range(4)])

    def transform_and_rate(self, t):
        m = self.transform_dual(t)
        return (np.array([[m[r][c].val for c in range(4)] for r in range(4)], dtype=np.float64),
                np.array([[m[r][c].grad for c in range(4)] for r in range(4)], dtype=np.float64))

    def transform_series(self, ts):
        """Transforms and rates at every time of ``ts``: two (len(ts), 4, 4) arrays."""
        ts = np.asarray(ts, np.float64)
        m = self.transform_dual_array(ts)
        val = np.empty((ts.size, 4, 4))
        grad = np.empty((ts.size, 4, 4))
        for r in range(4):
            for c in range(4):
                val[:, r, c] = np.broadcast_to(m[r][c].val, ts.shape)
                grad[:, r, c] = np.broadcast_to(m[r][c].grad, ts.shape)
        return val, grad

    def transform_dual_array(self, ts):
        own = self.fn(Dual(ts, np.ones_like(ts)))
        return matmul(self.parent.transform_dual_array(ts), own) if self.parent else own

    def linear_velocity(self, t, vertex):
        """d/dt of the transformed vertex (vlm_kinematics.hpp linear_velocity)."""
        _, d = self.transform_and_rate(t)
        return (d @ np.array([vertex[0], vertex[1], vertex[2], 1.0]))[:3]

    def angular_velocity(self, t):
        """vlm_kinematics.hpp angular_velocity: axial vector of Rdot R^T."""
        v, d = self.transform_and_rate(t)
        W = d[:3, :3] @ v[:3, :3].T
        return np.array([W[2, 1], W[0, 2], W[1, 0]])


class KinematicsTree:
    def __init__(self):
        self.nodes = []

    def placeholder(self):
        return self.add(None)

    def add(self, fn):
        n = KinematicNode(fn)
        self.nodes.append(n)
        return n


class Assembly:
    """vlm/include/vlm.hpp Assembly: surfaces with their kinematic nodes."""

    def __init__(self, assembly_node):
        self.node = assembly_node
        self.meshes, self.nodes, self.lifting = [], [], []

    def add(self, mesh, node, lifting=True):
        self.meshes.append(mesh)
        self.nodes.append(node)
        self.lifting.append(bool(lifting))

    def kinematics(self):
        return self.node

    def surface_kinematics(self):
        return self.nodes


def to_colmajor(m):
    return np.asarray(m, dtype=np.float64).T.ravel()
