"""JGSL: the Python module the Codim-IPC drivers import, backed by the GB300 path.

The reference's drivers (Python/Drivers/SimulationBase.py, FEMDiscreteShellBase.py)
do ``from JGSL import *`` and drive a simulation through pybind11 functions
(Library/EXPORTER.cpp:17-36; the shell module Library/FEM/Shell/DISCRETE_SHELL.h:
1085-1124).  This package provides those names with the same arguments, argument
meaning and in-place mutation, so that an unmodified driver runs on the GPU:

  * containers (Storage.*, StdVector*, StdMapPairiToi, CSR_MATRIX_D) and small
    vectors (Vector3d(...) etc., numpy arrays) hold the scene on the host, as
    the reference's containers do;
  * set-up (Add_Shell, Make_Rod, Add_Discrete_Particles, Initialize_*,
    Init_Dirichlet, MeshIO.*) runs on the host in Python, restating the
    reference's set-up routines (each cites its source);
  * FEM.DiscreteShell.Advance_One_Step_IE_Hinge (and its elastic-IPC and
    split-stepper variants) steps the scene with the C ABI (cipc_sim_step /
    cipc_sim_step_split): the first call creates the device-resident simulation
    from the containers; every call sends the positions, velocities, Dirichlet
    targets, kappa and kappa_s, steps, and writes positions, velocities, kappa
    (doubled when the barrier stiffness grows, as IMPLICIT_EULER.h:578-580 does
    to kappaVec) and kappa_s back into the driver's containers; it returns the
    Newton iteration count and appends the reference's residual.txt /
    counter.txt lines in the output folder.

What the GPU path does not implement raises NotImplementedError rather than
running something different: anisotropic membranes (fiberStiffMult != 0,
inextLimit != 0), per-component friction (muComp), static solves, stitching,
garments, normal flow, texture-mapped materials and 2D scenes.
"""
import math
import os
import sys

import numpy as np

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)
import cipc_ffi as _F  # noqa: E402

# ---------------------------------------------------------------------------
# runtime, parameters, timers (Library/Utils/PARAMETER.h, TIMER.h)
# ---------------------------------------------------------------------------
_PARAMS = {}


def Kokkos_Initialize(*args):
    """No host thread pool to start: the hot path runs on the GPU."""
    return None


def Kokkos_Finalize(*args):
    return None


def Set_Parameter(name, value):
    _PARAMS[name] = value


def Get_Parameter(name, default=None):
    return _PARAMS.get(name, default)


def TIMER_FLUSH(*args):
    """The reference prints its timer tree here; the GPU path reports per-step
    statistics in steps.jsonl instead."""
    return None


# ---------------------------------------------------------------------------
# scalars, vectors and matrices (Library/Math/VECTOR.h bindings): numpy arrays
# ---------------------------------------------------------------------------
Scalard = float
Scalarf = float


def _vec(n, dtype):
    def make(*a):
        if len(a) == 1 and np.ndim(a[0]) == 1:
            a = tuple(a[0])
        if not a:
            a = (0,) * n
        if len(a) != n:
            raise TypeError("expected %d components, got %d" % (n, len(a)))
        return np.array(a, dtype=dtype)
    return make


Vector2d, Vector3d, Vector4d = _vec(2, np.float64), _vec(3, np.float64), _vec(4, np.float64)
Vector2f, Vector3f, Vector4f = _vec(2, np.float32), _vec(3, np.float32), _vec(4, np.float32)
Vector2i, Vector3i, Vector4i = _vec(2, np.int64), _vec(3, np.int64), _vec(4, np.int64)


def Matrix2d(*a):
    return np.zeros((2, 2)) if not a else np.array(a, float).reshape(2, 2)


def Matrix3d(*a):
    return np.zeros((3, 3)) if not a else np.array(a, float).reshape(3, 3)


Matrix2f, Matrix3f = Matrix2d, Matrix3d

# ---------------------------------------------------------------------------
# containers (Library/Utils/STDCONTAINER.h:24-35, FEM_EXPORTER.h:15-49)
# ---------------------------------------------------------------------------


class _Rows:
    """A VECTOR_STORAGE / MESH_NODE / MESH_ELEM: rows of fixed width."""

    def __init__(self, width, dtype):
        self.a = np.zeros((0, width), dtype=dtype)

    @property
    def size(self):
        return self.a.shape[0]

    def __len__(self):
        return self.a.shape[0]

    def append_rows(self, rows):
        rows = np.asarray(rows, dtype=self.a.dtype).reshape(-1, self.a.shape[1])
        self.a = np.concatenate([self.a, rows], 0)

    def Get(self, i):
        return self.a[i].copy()

    def Copy(self):
        c = _Rows(self.a.shape[1], self.a.dtype)
        c.a = self.a.copy()
        return c


class _NodeAttr:
    """MESH_NODE_ATTR (x0, v, g, m) per node."""

    def __init__(self, dim=3):
        self.x0 = np.zeros((0, dim))
        self.v = np.zeros((0, dim))
        self.g = np.zeros((0, dim))
        self.m = np.zeros(0)

    @property
    def size(self):
        return self.v.shape[0]

    def resize(self, n, X):
        k = self.size
        if n > k:
            d = self.v.shape[1]
            self.x0 = np.concatenate([self.x0, X[k:n].copy()], 0)
            self.v = np.concatenate([self.v, np.zeros((n - k, d))], 0)
            self.g = np.concatenate([self.g, np.zeros((n - k, d))], 0)
            self.m = np.concatenate([self.m, np.zeros(n - k)], 0)


class _Motion(list):
    """DBC_MOTION: rows (range begin, range end, v, rotCenter, rotAxis, angVelDeg)."""

    @property
    def size(self):
        return len(self)


class _Opaque:
    """Containers whose content the GPU path keeps on the device (the element
    attributes, material and mass) or does not use."""

    def __init__(self, *a):
        self.args = a

    @property
    def size(self):
        return 0


class Storage:
    V2dStorage = staticmethod(lambda: _Rows(2, np.float64))
    V3dStorage = staticmethod(lambda: _Rows(3, np.float64))
    V4dStorage = staticmethod(lambda: _Rows(4, np.float64))
    V2iStorage = staticmethod(lambda: _Rows(2, np.int64))
    V3iStorage = staticmethod(lambda: _Rows(3, np.int64))
    V4iStorage = staticmethod(lambda: _Rows(4, np.int64))
    SiStorage = staticmethod(lambda: _Rows(1, np.int64))
    SdStorage = staticmethod(lambda: _Rows(1, np.float64))
    V2dV2dV2dSdStorage = staticmethod(lambda: _NodeAttr(2))
    V3dV3dV3dSdStorage = staticmethod(lambda: _NodeAttr(3))
    V2iV2dV2dV2dSdStorage = staticmethod(_Motion)
    V2iV3dV3dV3dSdStorage = staticmethod(_Motion)
    M2dM2dSdStorage = staticmethod(_Opaque)
    M3dM3dSdStorage = staticmethod(_Opaque)


class _StdVector(list):
    @property
    def size(self):
        return len(self)


def StdVectorXd(v=()):
    return _StdVector(float(a) for a in v)


def StdVectorXi(v=()):
    return _StdVector(int(a) for a in v)


StdVectorVector2i = StdVectorVector3i = StdVectorVector4i = StdVectorVector3d = _StdVector
StdMapPairiToi = dict


class CSR_MATRIX_D:
    """The driver's mass matrix.  Here it also carries the scene's set-up record
    and, after the first step, the device-resident simulation."""

    def __init__(self):
        self._scene = None


class _Elasticity:
    def __init__(self):
        self.E = None
        self.nu = None


class FIXED_COROTATED_2:
    Create = staticmethod(_Elasticity)


class FIXED_COROTATED_3:
    Create = staticmethod(_Elasticity)


# ---------------------------------------------------------------------------
# mesh IO (Library/Utils/MESHIO.h)
# ---------------------------------------------------------------------------


def _read_obj(path):
    V, F = [], []
    with open(path) as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "v":
                V.append([float(t[1]), float(t[2]), float(t[3])])
            elif t[0] == "f":
                F.append([int(s.split("/")[0]) - 1 for s in t[1:4]])
    return np.array(V, float).reshape(-1, 3), np.array(F, np.int64).reshape(-1, 3)


def _rotation(axis, deg, normalize):
    """Eigen::AngleAxis(angle, axis).toRotationMatrix(): c I + (1 - c) a a^T + s [a]x."""
    a = np.asarray(axis, float)
    if normalize:
        n = np.linalg.norm(a)
        a = a / n if n > 0 else a
    th = deg / 180 * math.pi
    c, s = math.cos(th), math.sin(th)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return c * np.eye(3) + (1 - c) * np.outer(a, a) + s * K


class MeshIO:
    @staticmethod
    def Read_TriMesh_Obj(path, X, Elem):
        """MESHIO.h Read_TriMesh_Obj: appends vertices and triangles; returns
        (first vertex, first triangle, vertex end, triangle end)."""
        V, F = _read_obj(path)
        c = Vector4i(X.size, Elem.size, X.size + V.shape[0], Elem.size + F.shape[0])
        F = F + X.size
        X.append_rows(V)
        Elem.append_rows(F)
        return c

    @staticmethod
    def Write_TriMesh_Obj(X, Elem, path):
        """MESHIO.h:182-213: "v %le %le %le" per node, "f i j k" (1-based)."""
        with open(path, "w") as f:
            for p in X.a:
                f.write("v %e %e %e\n" % (p[0], p[1], p[2]))
            for t in Elem.a:
                f.write("f %d %d %d\n" % (t[0] + 1, t[1] + 1, t[2] + 1))

    @staticmethod
    def Write_SegMesh_Obj(X, segs, path):
        with open(path, "w") as f:
            for p in X.a:
                f.write("v %e %e %e\n" % (p[0], p[1], p[2]))
            for s in segs:
                f.write("l %d %d\n" % (s[0] + 1, s[1] + 1))

    @staticmethod
    def Read_SegMesh_Seg(path, X, segs):
        V, S = [], []
        with open(path) as f:
            for line in f:
                t = line.split()
                if t and t[0] == "v":
                    V.append([float(t[1]), float(t[2]), float(t[3])])
                elif t and t[0] in ("l", "s"):
                    S.append([int(t[1]) - 1, int(t[2]) - 1])
        c = Vector4i(X.size, len(segs), X.size + len(V), len(segs) + len(S))
        for a, b in S:
            segs.append(Vector2i(a + X.size, b + X.size))
        X.append_rows(np.array(V, float).reshape(-1, 3))
        return c

    @staticmethod
    def Append_Attribute(src, dst):
        dst.append_rows(src.a)

    @staticmethod
    def Transform_Points(trans, rotCenter, rotAxis, rotDeg, scale, meshCounter, X):
        """MESHIO.h:837-869: x <- R (scale * (x - c)) + c + t on [counter[0], counter[2])."""
        R = _rotation(rotAxis, rotDeg, normalize=True)
        lo, hi = int(meshCounter[0]), int(meshCounter[2])
        x = (X.a[lo:hi] - rotCenter) * np.asarray(scale, float)
        X.a[lo:hi] = x @ R.T + rotCenter + trans

    @staticmethod
    def Load_Velocity(folder, lastFrame, h, nodeAttr):
        """MESHIO.h:967-984: v = (x(lastFrame) - x(lastFrame - 1)) / h."""
        x0, _ = _read_obj(os.path.join(folder, "%d.obj" % (lastFrame - 1)))
        x1, _ = _read_obj(os.path.join(folder, "%d.obj" % lastFrame))
        if x0.shape[0] != nodeAttr.size or x1.shape[0] != nodeAttr.size:
            raise ValueError("node count does not match")
        nodeAttr.v[:] = (x1 - x0) / h

    @staticmethod
    def Load_Velocity_X0(folder, lastFrame, h, X0, nodeAttr):
        x1, _ = _read_obj(os.path.join(folder, "%d.obj" % lastFrame))
        nodeAttr.v[:] = (x1 - X0.a) / h

    @staticmethod
    def Zero_Velocity(nodeAttr):
        nodeAttr.v[:] = 0


# ---------------------------------------------------------------------------
# scene set-up record and the device simulation behind it
# ---------------------------------------------------------------------------


class _Scene:
    def __init__(self):
        self.rho = self.E = self.nu = self.thickness = None
        self.gravity = np.array([0.0, -9.81, 0.0])
        self.rod = None  # (rod list, rho, E, thickness, bendMult)
        self.particles = None  # (particle list, rho, thickness)
        self.sim = None
        self.nv = 0
        self.ne = 0


def _scene(M):
    if M._scene is None:
        M._scene = _Scene()
    return M._scene


def _codim_desc(sc):
    if sc.rod is None and sc.particles is None:
        return None, []
    keep = []
    seg = np.zeros((0, 2), np.int32)
    par = np.zeros(0, np.int32)
    rE = rrho = rt = 0.0
    rb = 1.0
    prho = pt = 0.0
    if sc.rod is not None:
        rods, rrho, rE, rt, rb = sc.rod
        seg = np.ascontiguousarray(np.array([[int(a[0]), int(a[1])] for a in rods], np.int32).reshape(-1, 2))
    if sc.particles is not None:
        parts, prho, pt = sc.particles
        par = np.ascontiguousarray(np.array([int(p) for p in parts], np.int32))
    keep += [seg, par]
    d = _F.CodimDesc(seg.shape[0], seg.ctypes.data if seg.size else None, rE, rrho, rt, rb, par.shape[0],
                     par.ctypes.data if par.size else None, prho, pt)
    return d, keep


class FEM:
    class DiscreteShell:
        @staticmethod
        def Add_Shell(filePath, trans, scale, rotCenter, rotAxis, rotDeg, X, Elem, compNodeRange):
            """DISCRETE_SHELL.h Add_Discrete_Shell_3D: read an OBJ, map each node
            x -> R (scale * (x - c)) + c + t (R from the axis as given), append,
            record the component's node range; returns the counter."""
            V, F = _read_obj(filePath)
            R = _rotation(rotAxis, rotDeg, normalize=False)
            V = ((V - rotCenter) * np.asarray(scale, float)) @ R.T + rotCenter + trans
            c = Vector4i(X.size, Elem.size, X.size + V.shape[0], Elem.size + F.shape[0])
            Elem.append_rows(F + X.size)
            X.append_rows(V)
            compNodeRange.append(X.size)
            return c

        @staticmethod
        def Make_Rod(length, nSeg, X, rod):
            """Rod/DISCRETE_ROD.h:6-27: nSeg + 1 nodes along x, centred at 0."""
            c0, r0 = X.size, len(rod)
            xs = -length / 2 + np.arange(nSeg + 1) * (length / nSeg)
            X.append_rows(np.stack([xs, np.zeros_like(xs), np.zeros_like(xs)], 1))
            for i in range(nSeg):
                rod.append(Vector2i(c0 + i, c0 + i + 1))
            return Vector4i(c0, r0, X.size, len(rod))

        @staticmethod
        def Add_Discrete_Particles(length, num, randScale, X, particle, compNodeRange):
            """DISCRETE_PARTICLE.h:6-50: a num[0] x num[1] x num[2] lattice over
            `length`, each node jittered by randScale times a uniform draw in
            [-1, 1] per axis (drawn here from numpy's seeded generator, not the
            C library's rand(), so the jitter values differ)."""
            length = np.asarray(length, float)
            num = np.asarray(num, int)
            step = np.where(num > 1, length / np.maximum(num - 1, 1), length)
            rng = np.random.default_rng(0)
            c0, p0 = X.size, len(particle)
            pts = []
            for i in range(num[0]):
                for j in range(num[1]):
                    for k in range(num[2]):
                        r = rng.uniform(-1, 1, 3)
                        particle.append(X.size + len(pts))
                        pts.append(np.array([i, j, k]) * step + r * np.asarray(randScale, float))
            X.append_rows(np.array(pts, float).reshape(-1, 3))
            compNodeRange.append(X.size)
            return Vector4i(c0, p0, X.size, len(particle))

        @staticmethod
        def Initialize_Shell_Hinge_EIPC(rho0, E, nu, thickness, h, dHat2, X, Elem, seg, edge2tri, edgeStencil,
                                        edgeInfo, nodeAttr, M, gravity, b, elemAttr, elasticity, kappa):
            """DISCRETE_SHELL.h:218-357 (Initialize_Discrete_Shell): the shell's
            material and mass.  Recorded here; the device simulation built at the
            first step computes the mass, hinges and rest data on the host side of
            the C ABI (cipc_sim_create_full).  Returns dHat2."""
            sc = _scene(M)
            sc.X, sc.Elem = X, Elem
            sc.rho, sc.E, sc.nu, sc.thickness = float(rho0), float(E), float(nu), float(thickness)
            sc.gravity = np.asarray(gravity, float).copy()
            elasticity.E, elasticity.nu = float(E), float(nu)
            nodeAttr.resize(X.size, X.a)
            return dHat2

        @staticmethod
        def Initialize_Discrete_Rod(X, rod, rho0, E, thickness, gravity, b, nodeAttr, M, rodInfo, rodHinge,
                                    rodHingeInfo, bendStiffMult, h, dHat2, kappa):
            """Rod/DISCRETE_ROD.h:85-150: rods' material; mass, springs and hinges
            are built with the device simulation.  Returns dHat2."""
            sc = _scene(M)
            sc.rod = (list(rod), float(rho0), float(E), float(thickness), float(bendStiffMult))
            sc.gravity = np.asarray(gravity, float).copy()
            nodeAttr.resize(X.size, X.a)
            return dHat2

        @staticmethod
        def Initialize_Discrete_Particle(X, particle, rho0, E, thickness, gravity, b, nodeAttr, M):
            """DISCRETE_PARTICLE.h:52-75: particles' mass (4/3 pi t^3 / 8 rho)."""
            sc = _scene(M)
            sc.particles = (list(particle), float(rho0), float(thickness))
            sc.gravity = np.asarray(gravity, float).copy()
            nodeAttr.resize(X.size, X.a)

        @staticmethod
        def Initialize_OIPC(E, nu, thickness, h, M, kappa, stiffMult=1.0):
            """DISCRETE_SHELL.h:555-577 with elasticIPC = false: dHat = thickness;
            kappa[0] = stiffMult 1e11 mean(diag M) dim / (4e-16 b''(1e-16)),
            kappa[1] = 100 kappa[0] (computed by cipc_scene_oipc_kappa from the
            scene's lumped mass); returns dHat^2."""
            sc = _scene(M)
            X = sc.X
            kappa2, dhat2 = _F.scene_oipc_kappa(X.a, sc.Elem.a, sc.rho, sc.E, sc.nu, sc.thickness, sc.gravity,
                                                _codim_desc(sc)[0], float(thickness), float(stiffMult))
            kappa[0], kappa[1] = kappa2[0], kappa2[1]
            sc.kappa_init = True
            return dhat2

        @staticmethod
        def Initialize_EIPC(E, nu, thickness, h, M, kappa, stiffMult=1.0):
            """DISCRETE_SHELL.h:555-577 with elasticIPC = true: kappa = (h^2 mu,
            h^2 lambda, nu) of the plane-stress material, dHat^2 = thickness^2."""
            lam = E * nu / (1 - nu * nu)
            mu = E / (2 * (1 + nu))
            kappa[0], kappa[1], kappa[2] = h * h * mu, h * h * lam, nu
            return thickness * thickness

        @staticmethod
        def Advance_One_Step_IE_Hinge(Elem, segs, DBC, edge2tri, edgeStencil, edgeInfo, thickness,
                                      bendingStiffMult, fiberStiffMult, inextLimit, s, sHat, kappa_s, bodyForce, dt,
                                      PNTol, withCollision, dHat2, kappa, mu, epsv2, fricIterAmt, compNodeRange, muComp,
                                      staticSolve, X, nodeAttr, massMatrix, elemAttr, elasticity, tet, tetAttr,
                                      tetElasticity, rod, rodInfo, rodHinge, rodHingeInfo, stitchInfo, stitchRatio,
                                      k_stitch, discrete_particle, output_folder):
            """IMPLICIT_EULER.h:151-902 through cipc_sim_step; returns PNIter."""
            return _advance(False, False, locals())

        @staticmethod
        def Advance_One_Step_IE_Hinge_EIPC(Elem, segs, DBC, edge2tri, edgeStencil, edgeInfo, thickness,
                                           bendingStiffMult, fiberStiffMult, inextLimit, s, sHat, kappa_s, bodyForce,
                                           dt, PNTol, withCollision, dHat2, kappa, mu, epsv2, fricIterAmt,
                                           compNodeRange, muComp, staticSolve, X, nodeAttr, massMatrix, elemAttr,
                                           elasticity, tet, tetAttr, tetElasticity, rod, rodInfo, rodHinge,
                                           rodHingeInfo, stitchInfo, stitchRatio, k_stitch, discrete_particle,
                                           output_folder):
            """The elastic-IPC variant (DISCRETE_SHELL.h:1109-1110)."""
            return _advance(True, False, locals())

        @staticmethod
        def Advance_One_Step_SIE_Hinge(Elem, segs, DBC, edge2tri, edgeStencil, edgeInfo, thickness, bendingStiffMult,
                                       fiberStiffMult, inextLimit, s, sHat, kappa_s, bodyForce, dt, PNTol,
                                       withCollision, dHat2, kappa, mu, epsv2, fricIterAmt, compNodeRange, muComp,
                                       staticSolve, X, nodeAttr, massMatrix, elemAttr, elasticity, tet, tetAttr,
                                       tetElasticity, rod, rodInfo, rodHinge, rodHingeInfo, discrete_particle,
                                       output_folder):
            """The split stepper (SPLITTING_IE.h:362-729) through cipc_sim_step_split."""
            return _advance(False, True, locals())

        @staticmethod
        def Advance_One_Step_SIE_Hinge_EIPC(Elem, segs, DBC, edge2tri, edgeStencil, edgeInfo, thickness,
                                            bendingStiffMult, fiberStiffMult, inextLimit, s, sHat, kappa_s, bodyForce,
                                            dt, PNTol, withCollision, dHat2, kappa, mu, epsv2, fricIterAmt,
                                            compNodeRange, muComp, staticSolve, X, nodeAttr, massMatrix, elemAttr,
                                            elasticity, tet, tetAttr, tetElasticity, rod, rodInfo, rodHinge,
                                            rodHingeInfo, discrete_particle, output_folder):
            return _advance(True, True, locals())

        @staticmethod
        def _unsupported(name):
            def f(*a, **k):
                raise NotImplementedError("FEM.DiscreteShell.%s is not implemented by the GPU path" % name)
            return f

    @staticmethod
    def Init_Dirichlet(X, relBoxMin, relBoxMax, v, rotCenter, rotAxis, angVelDeg, DBC, DBCMotion,
                       vIndRange=(0, 0, 2 ** 31 - 1, -1)):
        """BOUNDARY_CONDITION.h:16-104: the nodes of [vIndRange[0], vIndRange[2])
        inside the box given relative to those nodes' bounding box become Dirichlet
        nodes (rows (index, x, y, z) of DBC, in index order), and the group gets a
        motion row (DBC range, v, rotCenter, rotAxis, angVelDeg)."""
        if X.size == 0:
            raise ValueError("no nodes in the model!")
        lo_i, hi_i = int(vIndRange[0]), min(int(vIndRange[2]), X.size)
        P = X.a[lo_i:hi_i]
        bmin, bmax = P.min(0), P.max(0)
        rmin = np.asarray(relBoxMin, float) * (bmax - bmin) + bmin
        rmax = np.asarray(relBoxMax, float) * (bmax - bmin) + bmin
        inside = np.all((P >= rmin) & (P <= rmax), 1)
        ring = float(Get_Parameter("Dirichlet_ring", 0.0))
        inside &= np.linalg.norm(P, axis=1) >= ring
        idx = np.nonzero(inside)[0] + lo_i
        begin = DBC.size
        DBC.append_rows(np.concatenate([idx[:, None].astype(float), X.a[idx]], 1))
        DBCMotion.append([begin, DBC.size, np.asarray(v, float).copy(), np.asarray(rotCenter, float).copy(),
                          np.asarray(rotAxis, float).copy(), float(angVelDeg)])

    @staticmethod
    def Step_Dirichlet(DBCMotion, h, DBC):
        """BOUNDARY_CONDITION.h:106-157: each group's targets are rotated by
        angVelDeg * pi / 180 * h about the axis (as given) through rotCenter,
        then moved by v h."""
        for begin, end, v, c, axis, ang in DBCMotion:
            if end <= begin:
                continue
            t = DBC.a[begin:end, 1:4]
            if ang != 0:
                R = _rotation(axis, ang * h, normalize=False)
                t = (t - c) @ R.T + c
            DBC.a[begin:end, 1:4] = t + np.asarray(v) * h

    @staticmethod
    def Turn_Dirichlet(DBCMotion):
        """BOUNDARY_CONDITION.h: reverse every group's velocity and rotation."""
        for row in DBCMotion:
            row[2] = -row[2]
            row[5] = -row[5]

    @staticmethod
    def Reset_Dirichlet(X, DBC):
        """Targets back to the nodes' current positions."""
        idx = DBC.a[:, 0].astype(np.int64)
        DBC.a[:, 1:4] = X.a[idx]

    @staticmethod
    def Pop_Back_Dirichlet(DBCMotion, DBC):
        """Drop the last Dirichlet node (and empty trailing groups)."""
        if DBC.size:
            DBC.a = DBC.a[:-1]
            for row in DBCMotion:
                row[1] = min(row[1], DBC.size)
                row[0] = min(row[0], row[1])


for _n in ("Add_Garment", "Initialize_Garment", "Make_Rod_Net", "Update_Normal_Flow_Neumann",
           "Update_Material_With_Tex_Shell", "Adjust_Material", "Advance_One_Step_IE_Flow"):
    setattr(FEM.DiscreteShell, _n, staticmethod(FEM.DiscreteShell._unsupported(_n)))


def _fem_unsupported(name):
    def f(*a, **k):
        raise NotImplementedError("FEM.%s is not implemented by the GPU path" % name)
    return f


for _n in ("Load_Dirichlet", "Boundary_Dirichlet", "Magnify_Body_Force", "Update_Inv_Basis",
           "Compute_Vol_And_Inv_Basis", "Compute_Mass_And_Init_Velocity_NoAlloc",
           "Augment_Mass_Matrix_And_Body_Force"):
    setattr(FEM, _n, staticmethod(_fem_unsupported(_n)))


def _check_supported(a):
    if np.any(np.asarray(a["fiberStiffMult"], float) != 0) or np.any(np.asarray(a["inextLimit"], float) != 0):
        raise NotImplementedError("anisotropic membranes (fiberStiffMult, inextLimit) are not implemented by the "
                                  "GPU path")
    if len(a["muComp"]) and not np.all(np.asarray(a["muComp"], float) == float(a["mu"])):
        raise NotImplementedError("per-component friction (muComp) is not implemented by the GPU path")
    if a["staticSolve"]:
        raise NotImplementedError("static solves are not implemented by the GPU path")
    if len(a.get("stitchInfo", ())):
        raise NotImplementedError("stitching is not implemented by the GPU path")
    if getattr(a["tet"], "size", 0):
        raise NotImplementedError("volumetric tets through this driver entry are not wired (use cipc_sim_create_full)")


def _advance(elastic, split, a):
    """Steps the driver's scene once on the GPU and writes the results back into
    its containers; returns the Newton iteration count."""
    _check_supported(a)
    M, X, Elem, nodeAttr, DBC = a["massMatrix"], a["X"], a["Elem"], a["nodeAttr"], a["DBC"]
    sc = _scene(M)
    if sc.sim is None:
        if sc.rho is None:
            raise RuntimeError("Initialize_Shell_Hinge_EIPC was not called for this scene")
        cd, keep = _codim_desc(sc)
        sc.keep = keep
        sc.sim = _F.Sim(X.a, Elem.a, sc.rho, sc.E, sc.nu, sc.thickness, gravity=tuple(sc.gravity),
                        bend_stiff_mult=float(a["bendingStiffMult"]), nh=True,
                        codim=None if cd is None else dict(
                            segments=keep[0], particles=keep[1],
                            rod_E=cd.rod_E, rod_rho=cd.rod_rho, rod_thickness=cd.rod_thickness,
                            rod_bend_mult=cd.rod_bend_mult, particle_rho=cd.particle_rho,
                            particle_thickness=cd.particle_thickness))
        sc.nv = X.size
    sim = sc.sim
    if X.size != sc.nv:
        raise RuntimeError("the scene's node count changed after the first step")
    nodeAttr.resize(X.size, X.a)
    sim.set_state(X.a, nodeAttr.v)
    kappa = a["kappa"]
    if not elastic:
        sim.set_kappa(float(kappa[0]), float(kappa[1]))
    s, sHat, kappa_s = a["s"], a["sHat"], a["kappa_s"]
    sim.set_strain_limit(s, sHat, kappa_s)
    idx = DBC.a[:, 0].astype(np.int32) if DBC.size else np.zeros(0, np.int32)
    sim.set_dbc(idx, DBC.a[:, 1:4] if DBC.size else np.zeros((0, 3)))
    out = a["output_folder"]
    if out:
        os.makedirs(out, exist_ok=True)
        _F.sim_set_output(sim, out)
    # the GPU path's own choices, set by Set_Parameter: precision ("fp64" or
    # "mixed") and preconditioner (0 block Jacobi, 2 aggregate block Jacobi)
    prec = _F.MIXED if str(Get_Parameter("cipc_precision", "fp64")) == "mixed" else _F.FP64
    pre = int(Get_Parameter("cipc_preconditioner", _F.PRECOND_BLOCK_JACOBI))
    prm = _F.make_params(float(a["dt"]), float(a["dHat2"]), float(a["thickness"]), mu=float(a["mu"]),
                         epsv2=float(a["epsv2"]), fric_iters=int(a["fricIterAmt"]), newton_tol=float(a["PNTol"]),
                         with_collision=bool(a["withCollision"]), elastic_ipc=elastic, precision=prec,
                         preconditioner=pre)
    if elastic:
        sim.set_kappa(float(kappa[0]), float(kappa[0]))
    st = (sim.step_split if split else sim.step)(prm, allow=(_F.CIPC_ERR_NOT_CONVERGED,))
    x, v = sim.state()
    X.a[:] = x
    nodeAttr.v[:] = v
    if not elastic:
        k2 = sim.kappa()
        kappa[0], kappa[1] = k2[0], k2[1]
    ks = sim.strain_kappa()
    kappa_s[0], kappa_s[1] = ks[0], ks[1]
    return int(st.newton_iters)


__all__ = [n for n in dir() if not n.startswith("_") and n not in ("math", "os", "sys", "np")]
