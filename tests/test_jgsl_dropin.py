"""The JGSL module behind the reference's own Python drivers.

CPU test (here, where the Codim-IPC sources are present): the reference's
unmodified driver package (Python/Drivers: SimulationBase.py,
FEMDiscreteShellBase.py) is imported with this repository's JGSL on the path and
set up a 40x40 cloth over a fixed cube exactly as its scene scripts do
(add_shell_3D, set_DBC, initialize, initialize_OIPC).  Every JGSL name the
drivers reference at module level resolves; the set-up fills the driver's
containers (nodes, triangles, Dirichlet rows) and kappa equals the oracle's
Initialize_OIPC value; a time step reaches FEM.DiscreteShell.
Advance_One_Step_IE_Hinge with the driver's 40 arguments and, without a GPU,
fails loudly (CIPC_ERR_NO_DEVICE: there is no CPU fallback).

GPU test (on the GB300, where the reference is not present): the same call
sequence the driver makes, through JGSL, steps the scene three times; positions
and velocities match a direct cipc_sim_step run of the same scene.
"""
import io
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "codim-ipc_gb300")
sys.path.insert(0, ROOT)
from oracle.build import REF_ROOT  # noqa: E402  (where the oracle's build recipe finds the reference)

REF_PY = os.path.join(REF_ROOT, "Python")


def _write_obj(path, X, T):
    with open(path, "w") as f:
        for p in X:
            f.write("v %.17g %.17g %.17g\n" % tuple(p))
        for t in T:
            f.write("f %d %d %d\n" % (t[0] + 1, t[1] + 1, t[2] + 1))


def _scene_files(d):
    import workloads as W
    cl_X, cl_T = W.cloth_grid(40, 40, 1.0, 1.0, y=0.0, origin=(-0.5, -0.5))
    bx_X, bx_T = W.box_shell(0.3, (0.0, -0.1 - 0.15, 0.0), 4)
    _write_obj(os.path.join(d, "cube.obj"), bx_X, bx_T)
    _write_obj(os.path.join(d, "cloth.obj"), cl_X, cl_T)
    return cl_X, cl_T, bx_X, bx_T


def _set_up(sim, d, Vector3d):
    sim.add_shell_3D(os.path.join(d, "cube.obj"), Vector3d(0, 0, 0), Vector3d(0, 0, 0), Vector3d(0, 1, 0), 0)
    sim.set_DBC(Vector3d(-0.1, -0.1, -0.1), Vector3d(1.1, 1.1, 1.1), Vector3d(0, 0, 0), Vector3d(0, 0, 0),
                Vector3d(0, 1, 0), 0)
    sim.add_shell_3D(os.path.join(d, "cloth.obj"), Vector3d(0, 0, 0), Vector3d(0, 0, 0), Vector3d(0, 1, 0), 0)
    sim.dt = 0.04
    sim.frame_dt = 0.04
    sim.frame_num = 3
    sim.withCollision = True
    sim.PNTol = 1e-2
    sim.initialize(200.0, 1e5, 0.3, 1e-3, 0)
    sim.initialize_OIPC(1e-3, 1e-3)


@pytest.mark.skipif(not os.path.isdir(REF_PY + "/Drivers"), reason="the reference's drivers are not present")
def test_unmodified_reference_driver_runs_on_jgsl(tmp_path, monkeypatch, orc):
    monkeypatch.chdir(tmp_path)
    monkeypatch.setattr(sys, "argv", ["cloth_on_cube.py"])
    for p in (REF_PY, PKG):
        monkeypatch.syspath_prepend(p)
    for m in [m for m in sys.modules if m == "Drivers" or m.startswith("Drivers.") or m == "JGSL"]:
        monkeypatch.delitem(sys.modules, m)
    stdout = sys.stdout
    try:
        import Drivers
        import JGSL
        assert JGSL.__file__.startswith(PKG)  # this repository's module, not a build of the reference
        cl_X, cl_T, bx_X, bx_T = _scene_files(str(tmp_path))
        sim = Drivers.FEMDiscreteShellBase("double", 3)
        _set_up(sim, str(tmp_path), JGSL.Vector3d)
        nv = bx_X.shape[0] + cl_X.shape[0]
        assert sim.X.size == nv and sim.Elem.size == bx_T.shape[0] + cl_T.shape[0]
        assert sim.DBC.size == bx_X.shape[0] and np.array_equal(sim.DBC.a[:, 0], np.arange(bx_X.shape[0]))
        # kappa from the scene's lumped mass, as Initialize_OIPC computes it
        X = np.concatenate([bx_X, cl_X])
        T = np.concatenate([bx_T, cl_T + bx_X.shape[0]])
        k2_o, d2_o = orc.Shell(X, T, 200.0, 1e5, 0.3, 1e-3).init_oipc(1e-3)
        assert sim.dHat2 == d2_o
        assert np.allclose(sim.kappa[:2], k2_o, rtol=1e-12)
        import cipc_ffi as F
        if F.lib().cipc_device_count() == 0:
            with pytest.raises(F.CipcError) as ei:
                sim.advance_one_time_step(sim.dt)
            assert ei.value.status == F.CIPC_ERR_NO_DEVICE
    finally:
        sys.stdout = stdout


def test_jgsl_covers_the_drivers_names():
    """Every JGSL name the reference's shell driver calls is defined (checked on
    the module, no reference needed: the list is the driver's call sites)."""
    sys.path.insert(0, PKG)
    import JGSL
    names = ["Kokkos_Initialize", "Set_Parameter", "Get_Parameter", "TIMER_FLUSH", "Scalard", "Vector2d", "Vector3d",
             "Vector4d", "Vector4i", "Matrix3d", "StdVectorVector2i", "StdVectorXd", "StdVectorXi", "StdMapPairiToi",
             "StdVectorVector4i", "StdVectorVector3d", "StdVectorVector3i", "CSR_MATRIX_D", "FIXED_COROTATED_2",
             "FIXED_COROTATED_3"]
    for n in names:
        assert hasattr(JGSL, n), n
    for n in ("V3dStorage", "V3iStorage", "V4dStorage", "V3dV3dV3dSdStorage", "V2iV3dV3dV3dSdStorage",
              "M2dM2dSdStorage", "M3dM3dSdStorage", "V4iStorage", "SiStorage", "SdStorage"):
        assert hasattr(JGSL.Storage, n), n
    for n in ("Add_Shell", "Make_Rod", "Add_Discrete_Particles", "Initialize_Shell_Hinge_EIPC",
              "Initialize_Discrete_Rod", "Initialize_Discrete_Particle", "Initialize_OIPC", "Initialize_EIPC",
              "Advance_One_Step_IE_Hinge", "Advance_One_Step_IE_Hinge_EIPC", "Advance_One_Step_SIE_Hinge",
              "Advance_One_Step_SIE_Hinge_EIPC"):
        assert callable(getattr(JGSL.FEM.DiscreteShell, n)), n
    for n in ("Init_Dirichlet", "Step_Dirichlet", "Turn_Dirichlet", "Reset_Dirichlet", "Pop_Back_Dirichlet"):
        assert callable(getattr(JGSL.FEM, n)), n
    for n in ("Read_TriMesh_Obj", "Write_TriMesh_Obj", "Append_Attribute", "Transform_Points", "Load_Velocity",
              "Write_SegMesh_Obj", "Read_SegMesh_Seg", "Zero_Velocity"):
        assert callable(getattr(JGSL.MeshIO, n)), n


def test_dirichlet_motion_matches_device_restatement():
    """JGSL's host Init_Dirichlet / Step_Dirichlet rotate and translate targets as
    the reference does: a quarter turn about y over 0.5 s at 180 deg/s."""
    sys.path.insert(0, PKG)
    import JGSL as J
    X = J.Storage.V3dStorage()
    X.append_rows([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [2.0, 0.5, 0.0]])
    DBC, mot = J.Storage.V4dStorage(), J.Storage.V2iV3dV3dV3dSdStorage()
    J.FEM.Init_Dirichlet(X, J.Vector3d(-0.1, -0.1, -0.1), J.Vector3d(0.6, 1.1, 1.1), J.Vector3d(0, 0, 0),
                         J.Vector3d(0, 0, 0), J.Vector3d(0, 1, 0), 180.0, DBC, mot)
    assert list(DBC.a[:, 0]) == [0.0, 1.0]
    J.FEM.Step_Dirichlet(mot, 0.5, DBC)
    assert np.allclose(DBC.a[0, 1:], [0.0, 0.0, -1.0], atol=1e-15)
    assert np.allclose(DBC.a[1, 1:], [0.0, 1.0, 0.0])


@pytest.mark.gpu
def test_driver_call_sequence_steps_on_gpu(cuda, tmp_path):
    sys.path.insert(0, PKG)
    import cipc_ffi as F
    import JGSL as J
    cl_X, cl_T, bx_X, bx_T = _scene_files(str(tmp_path))

    class Driver:  # the attributes FEMDiscreteShellBase keeps, with its defaults
        def __init__(self):
            self.X, self.Elem = J.Storage.V3dStorage(), J.Storage.V3iStorage()
            self.segs, self.compNodeRange = J.StdVectorVector2i(), J.StdVectorXi()
            self.nodeAttr, self.massMatrix = J.Storage.V3dV3dV3dSdStorage(), J.CSR_MATRIX_D()
            self.elemAttr, self.elasticity = J.Storage.M2dM2dSdStorage(), J.FIXED_COROTATED_2.Create()
            self.DBC, self.DBCMotion = J.Storage.V4dStorage(), J.Storage.V2iV3dV3dV3dSdStorage()
            self.gravity, self.bodyForce = J.Vector3d(0, -9.81, 0), J.StdVectorXd()
            self.kappa, self.s, self.sHat, self.kappa_s = J.Vector3d(1e5, 0, 0), J.Vector2d(1.01, 0), \
                J.Vector2d(1, 1), J.Vector2d(0, 0)
            self.dt, self.dHat2, self.output_folder = 0.04, 1e-6, str(tmp_path) + "/"

        def add_shell_3D(self, path, t, c, a, deg):
            return J.FEM.DiscreteShell.Add_Shell(path, t, J.Vector3d(1, 1, 1), c, a, deg, self.X, self.Elem,
                                                 self.compNodeRange)

        def step(self):
            J.FEM.Step_Dirichlet(self.DBCMotion, self.dt, self.DBC)
            return J.FEM.DiscreteShell.Advance_One_Step_IE_Hinge(
                self.Elem, self.segs, self.DBC, J.StdMapPairiToi(), J.StdVectorVector4i(), J.StdVectorVector3d(),
                self.thickness, 1, J.Vector4d(0, 0, 0, 0), J.Vector3d(0, 0, 0), self.s, self.sHat, self.kappa_s,
                self.bodyForce, self.dt, 1e-2, True, self.dHat2, self.kappa, 0.0, 1e-6, 1, self.compNodeRange,
                J.StdVectorXd(), False, self.X, self.nodeAttr, self.massMatrix, self.elemAttr, self.elasticity,
                J.Storage.V4iStorage(), J.Storage.M3dM3dSdStorage(), J.FIXED_COROTATED_3.Create(),
                J.StdVectorVector2i(), J.StdVectorVector3d(), J.StdVectorVector3i(), J.StdVectorVector3d(),
                J.StdVectorVector3i(), J.StdVectorXd(), 10, J.StdVectorXi(), self.output_folder)

    drv = Driver()
    drv.add_shell_3D(str(tmp_path / "cube.obj"), J.Vector3d(0, 0, 0), J.Vector3d(0, 0, 0), J.Vector3d(0, 1, 0), 0)
    J.FEM.Init_Dirichlet(drv.X, J.Vector3d(-0.1, -0.1, -0.1), J.Vector3d(1.1, 1.1, 1.1), J.Vector3d(0, 0, 0),
                         J.Vector3d(0, 0, 0), J.Vector3d(0, 1, 0), 0, drv.DBC, drv.DBCMotion)
    drv.add_shell_3D(str(tmp_path / "cloth.obj"), J.Vector3d(0, 0, 0), J.Vector3d(0, 0, 0), J.Vector3d(0, 1, 0), 0)
    drv.dHat2 = J.FEM.DiscreteShell.Initialize_Shell_Hinge_EIPC(
        200.0, 1e5, 0.3, 1e-3, drv.dt, drv.dHat2, drv.X, drv.Elem, drv.segs, J.StdMapPairiToi(),
        J.StdVectorVector4i(), J.StdVectorVector3d(), drv.nodeAttr, drv.massMatrix, drv.gravity, drv.bodyForce,
        drv.elemAttr, drv.elasticity, drv.kappa)
    drv.dHat2 = J.FEM.DiscreteShell.Initialize_OIPC(0.0, 0.0, 1e-3, 0.0, drv.massMatrix, drv.kappa, 1)
    drv.thickness = 1e-3
    X0 = drv.X.a.copy()
    T = drv.Elem.a.copy()
    its = [drv.step() for _ in range(3)]
    assert all(i > 0 for i in its)
    # the same scene stepped directly through the C ABI
    s = F.Sim(X0, T, 200.0, 1e5, 0.3, 1e-3)
    _, dhat2 = s.init_oipc(1e-3)
    dbc = np.arange(bx_X.shape[0], dtype=np.int32)
    prm = F.make_params(0.04, dhat2, 1e-3, newton_tol=1e-2)
    for _ in range(3):
        s.set_dbc(dbc, X0[dbc])
        s.step(prm)
    x, v = s.state()
    diag = np.linalg.norm(X0.max(0) - X0.min(0))
    assert np.abs(drv.X.a - x).max() <= 1e-9 * diag
    assert np.abs(drv.nodeAttr.v - v).max() <= 1e-9 * diag / 0.04
    assert (tmp_path / "counter.txt").exists() and len((tmp_path / "counter.txt").read_text().splitlines()) == 3
    s.close()
