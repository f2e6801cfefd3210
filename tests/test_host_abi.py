"""CPU tests of the C-ABI library: it loads and exports every entry point include/af3d.h
declares, and its host-only parts (DataInput.dat, derived parameters, error_check,
last_config.dat, initial-state generators) match the reference.  No GPU call is made."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def af3d():
    from avalancheflume3d_gb300 import build
    build.build()
    import avalancheflume3d_gb300 as af3d
    af3d.lib()
    return af3d


def _declared_symbols():
    src = open(os.path.join(ROOT, "include", "af3d.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(af3d_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(af3d):
    import subprocess
    names = _declared_symbols()
    assert len(names) >= 50
    out = subprocess.run(["nm", "-D", "--defined-only", af3d.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (af3d_[a-z0-9_]+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    from avalancheflume3d_gb300._lib import SIGNATURES
    bound = {s[0] for s in SIGNATURES}
    assert set(names) <= bound, sorted(set(names) - bound)
    assert af3d.lib().af3d_abi_version() == 1


def test_struct_sizes_match_reference(reference):
    from avalancheflume3d_gb300 import PARTICLE, SYSTEM_PAR, CELL_PAR
    assert reference.lib.ref_sizeof_particle() == PARTICLE.itemsize == 408
    assert reference.lib.ref_sizeof_system_par() == SYSTEM_PAR.itemsize == 256
    assert reference.lib.ref_sizeof_cell_par() == CELL_PAR.itemsize == 168


DATAINPUT = """20358       Number of particles.
15.0        Flume and width.
75.0        Hopper height.
0.17979588  Minimum sphere radius.
0.17979588  Maximum sphere radius.
10.0        Initial velocity.
1.0e-6      Time step.
0.6         Particle-wall coefficient of restitution.
0.4         Particle-wall coefficient of friction.
0.6         Particle-particle coefficient of restitution.
0.4         Particle-particle coefficient of friction.
1.0e-4      Collision time.
140.0       Flume length.
35.0        Flume tilt in degrees.
9           Number of tagged particles in cells.
1           Print flag.
All values are in cgs units.
"""


def test_datainput_parse_and_derive(af3d, tmp_path):
    from oracle.pyoracle import make_system
    p = tmp_path / "DataInput.dat"
    p.write_text(DATAINPUT)
    v = af3d.load_datainput(str(p))
    assert int(v["npart"]) == 20358 and int(v["ntags"]) == 9 and int(v["print_flag"]) == 1
    assert float(v["rmin"]) == 0.17979588 and float(v["t_coll"]) == 1.0e-4 and float(v["tilt_deg"]) == 35.0
    sys, fun = af3d.derive_system(v)
    ref_sys, ref_fun = make_system(20358, 15.0, 75.0, 0.17979588, 0.17979588, 10.0, 1.0e-6, 0.6, 0.4,
                                   0.6, 0.4, 1.0e-4, 140.0, 35.0, time=-1.0)
    assert sys.tobytes() == ref_sys.tobytes()
    assert fun.tobytes() == ref_fun.tobytes()


def test_datainput_errors(af3d, tmp_path):
    p = tmp_path / "short.dat"
    p.write_text("\n".join(DATAINPUT.splitlines()[:10]))
    with pytest.raises(af3d.EngineError) as e:
        af3d.load_datainput(str(p))
    assert e.value.code == 8
    with pytest.raises(af3d.EngineError):
        af3d.load_datainput(str(tmp_path / "missing.dat"))


@pytest.mark.parametrize("case", range(8))
def test_error_check_matches_reference(af3d, reference, case):
    from oracle.pyoracle import make_system
    sys, _ = make_system(100, 15.0, 75.0, 0.18, 0.18, 10.0, 1e-6, 0.6, 0.4, 0.6, 0.4, 1e-4, 140.0, 35.0)
    edits = [{}, {"npart": 0}, {"rmin": -1.0}, {"rmax": 0.1}, {"eps_pw": 1.5}, {"mu_pp": 2.0},
             {"mu_pw": 0.7}, {"tilt": 0.2}]
    for k, v in edits[case].items():
        sys[k] = v
    got, msg = af3d.error_check(sys)
    assert got == reference.error_check(sys)
    assert (got == 0) == (msg == "")


def test_rannew64_and_generators_match_reference(af3d, reference):
    from oracle.pyoracle import make_system
    idum = np.array([26752658], dtype=np.int64)
    want = [reference.rannew64(idum) for _ in range(600)]
    r = af3d.Rannew64(26752658)
    assert [r() for _ in range(600)] == want
    n = 700
    sys, _ = make_system(n, 15.0, 75.0, 0.16, 0.18, 10.0, 1e-6, 0.6, 0.4, 0.6, 0.4, 1e-4, 140.0, 35.0)
    sys["side"][0] = 15.0
    ours = af3d.generate_particles(sys)
    theirs = np.zeros(n, dtype=ours.dtype)
    reference.lib.ref_generate_particles(theirs.ctypes.data, sys.ctypes.data)
    af3d.calculate_particle_parameters(ours)
    reference.lib.ref_calculate_particle_parameters_hst(sys.ctypes.data, theirs.ctypes.data)
    af3d.place_particles(sys, ours)
    reference.lib.ref_place_particles(sys.ctypes.data, theirs.ctypes.data)
    # set_initial_velocity re-seeds; the reference's generator is already seeded with the same idum
    # (its state persists), so compare against a fresh restatement of the same sequence instead.
    af3d.set_initial_velocity(sys, ours)
    for f in ("radius", "density", "mass", "moment_of_inertia", "rr", "rr_s", "Rmatx", "Rmaty", "Rmatz"):
        assert ours[f].tobytes() == theirs[f].tobytes(), f
    rr = af3d.Rannew64(26752658)
    r0 = 2.0 * 3.1415926535897932 * rr() - 3.1415926535897932
    r1 = 3.1415926535897932 * rr()
    assert ours["vv"][0, 2] == float(sys["v0"]) * np.sin(r1)


def test_set_initial_velocity_matches_reference_fresh_process(af3d, tmp_path):
    """The reference's rannew64 keeps static state, so its set_initial_velocity is compared in a
    fresh process where it is the first draw, as in the reference's start-up."""
    import subprocess
    import sys as _sys
    code = r'''
import sys, numpy as np
sys.path.insert(0, %r)
from oracle.pyoracle import Reference, make_system, PARTICLE
import avalancheflume3d_gb300 as af3d
ref = Reference()
s, _ = make_system(500, 15.0, 75.0, 0.18, 0.18, 10.0, 1e-6, 0.6, 0.4, 0.6, 0.4, 1e-4, 140.0, 35.0)
a = np.zeros(500, dtype=PARTICLE); b = np.zeros(500, dtype=PARTICLE)
ref.lib.ref_set_initial_velocity(s.ctypes.data, a.ctypes.data)
af3d.set_initial_velocity(s, b)
print(a["vv"].tobytes() == b["vv"].tobytes() and a["ww"].tobytes() == b["ww"].tobytes())
''' % ROOT
    from oracle import build
    if not build.reference_available():
        pytest.skip("reference tree absent")
    out = subprocess.run([_sys.executable, "-c", code], capture_output=True, text=True)
    assert out.stdout.strip() == "True", out.stdout + out.stderr


def test_last_config_round_trip(af3d, tmp_path):
    from oracle.pyoracle import dense_state
    from tests.states import flume_system
    n = 50
    sys, _ = flume_system(n)
    pp = dense_state(n, 1, sys)
    path = str(tmp_path / "last_config.dat")
    af3d.write_last_config(path, pp, 1, 0.123456789, 20001, 3)
    q = np.zeros(n, dtype=pp.dtype)
    q["radius"] = pp["radius"]
    head = af3d.read_last_config(path, q)
    assert head[0] == 1 and abs(head[1] - 0.123457) < 1e-12 and head[2:] == (20001, 3)
    for f in ("rr", "vv", "ww", "Rmatx"):
        assert np.max(np.abs(q[f] - pp[f])) <= 5e-7      # %lf keeps 6 decimals (lossy, as the reference)
    text = open(path).read().splitlines()
    assert text[:4] == ["1", "0.123457", "20001", "3"] and len(text) == 4 + n


@pytest.mark.parametrize("phase", [0, 1])
def test_snapshot_frames_in_the_reference_format(af3d, tmp_path, phase):
    """af3d_append_snapshot writes the frames of avalanche_hst.cu:507-586 (fill phase) and
    :750-841 (avalanche phase): the same format strings, the same ghost atoms, the same sums."""
    import math
    from oracle.pyoracle import dense_state
    from tests.states import flume_system
    n = 7
    sys, _ = flume_system(n, time=0.25 if phase == 1 else -0.5)
    pp = dense_state(n, 3, sys)
    pp["vv"] = np.random.default_rng(1).standard_normal((n, 3))
    pp["ww"] = np.random.default_rng(2).standard_normal((n, 3))
    sys["tot_mass"] = float(np.sum(pp["mass"]))
    paths = {k: str(tmp_path / (k + ".out")) for k in ("xyz", "vel", "vmean", "xcm")}
    for _ in range(2):   # two frames appended
        af3d.append_snapshot(pp, sys, phase, **paths)
    xfinal = (70.0 + float(sys["Lflume"])) * float(sys["cost"])
    side = sys["side"]
    want_xyz = ["%d" % (4 * n + 2), ""]
    for i in range(n):
        for k in range(4):
            want_xyz.append("%f %f %f %f %d" % (pp["radius"][i], *pp["rr_s"][i][k], i))
    if phase == 1:
        want_xyz.append("0.0001 %f %f %f %d" % (side[0], 30.0, side[2], n))
    else:
        want_xyz.append("0.000001 %f %f %f %d" % (xfinal, 30.0, side[2], n))
    want_xyz.append("0.000001 0.000000 0.000000 0.000000 %d" % n)
    assert open(paths["xyz"]).read().splitlines() == want_xyz * 2
    want_vel = ["%d" % (n + 2), ""]
    for i in range(n):
        want_vel.append("%f %f %f %f %f %d" % (*pp["rr"][i], pp["vv"][i][0], pp["ww"][i][1], i))
    want_vel.append("%f %f %f 0.000000 0.000000 %d" % (xfinal, 30.0, side[2], n))
    want_vel.append("0.000000 0.000000 0.000000 0.000000 0.000000 %d" % n)
    assert open(paths["vel"]).read().splitlines() == want_vel * 2
    vm = sum(math.sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]) for v in pp["vv"]) / n
    wm = sum(math.sqrt((w[0] * w[0] + w[1] * w[1]) + w[2] * w[2]) for w in pp["ww"]) / n
    t = float(sys["time"]) - float(sys["dt"])
    assert open(paths["vmean"]).read().splitlines() == ["%f, %f, %f" % (t, vm, wm)] * 2
    if phase == 1:
        xcm = sum(pp["mass"][i] * pp["rr"][i][0] for i in range(n)) / float(sys["tot_mass"])
        zcm = sum(pp["mass"][i] * pp["rr"][i][2] for i in range(n)) / float(sys["tot_mass"])
        assert open(paths["xcm"]).read().splitlines() == ["%f, %f, %f" % (t, xcm, zcm)] * 2
    else:
        import os
        assert not os.path.exists(paths["xcm"])   # the fill phase writes no centre of mass


def test_lattice_block_workload(af3d):
    from avalancheflume3d_gb300.workloads import flume_2k, flume_state
    sys, fun, pp = flume_state(flume_2k())
    assert len(pp) == 2048 and np.all(pp["rr"][:, 2] > 25.0)
    # no sphere overlaps and every sphere inside the hopper box
    s = pp["rr_s"].reshape(-1, 3)
    assert s[:, 0].min() >= pp["radius"][0] - 1e-12 and s[:, 0].max() <= 15.0 - pp["radius"][0] + 1e-12
    R = np.stack([pp["Rmatx"], pp["Rmaty"], pp["Rmatz"]], 1)
    assert np.allclose(np.einsum("nij,nkj->nik", R, R), np.eye(3), atol=1e-12)
    again = flume_state(flume_2k())[2]
    assert again.tobytes() == pp.tobytes()


def test_bed_layer_workload(af3d):
    """The dense layer on the flume bed: every sphere above the bed plane and between the side
    walls (slope frame), rotations orthonormal, and resting contacts only (overlaps at rounding
    level, no interpenetration)."""
    from avalancheflume3d_gb300.workloads import flume_2k, flume_state
    sys, fun, pp = flume_state(flume_2k(n=3000, layout="bed"))
    r = float(pp["radius"][0])
    q = pp["rrot_s"].reshape(-1, 3)
    dy2, width = float(sys["dy2"]), float(sys["side"][1])
    assert q[:, 2].min() >= r - 1e-9                      # on or above the bed z' = 0
    assert q[:, 1].min() >= dy2 + r - 1e-9 and q[:, 1].max() <= dy2 + width - r + 1e-9
    assert q[:, 0].min() >= 71.0 + r - 1e-9 and q[:, 0].max() <= 109.0 - r + 1e-9
    R = np.stack([pp["Rmatx"], pp["Rmaty"], pp["Rmatz"]], 1)
    assert np.allclose(np.einsum("nij,nkj->nik", R, R), np.eye(3), atol=1e-12)
    # sphere pairs of different clumps: separation >= 2r up to rounding
    from scipy.spatial import cKDTree
    owner = np.repeat(np.arange(len(pp)), 4)
    pairs = cKDTree(q).query_pairs(2 * r - 1e-9, output_type="ndarray")
    pairs = pairs[owner[pairs[:, 0]] != owner[pairs[:, 1]]]
    assert len(pairs) == 0
    touching = cKDTree(q).query_pairs(2 * r + 1e-9, output_type="ndarray")
    assert len(touching) > len(pp) // 2                    # a packed layer, not a loose lattice


def test_ensemble_configs_draws(af3d):
    from avalancheflume3d_gb300.workloads import ensemble_configs, ensemble_flagged, ensemble_state
    cfgs = ensemble_configs(256)
    n = np.array([c.n for c in cfgs])
    assert n.min() >= 1024 and n.max() <= 16384 and len(set(n.tolist())) > 200
    for name, lo, hi in (("mu_pp", 0.2, 0.8), ("mu_pw", 0.2, 0.6), ("restitution", 0.2, 0.8),
                         ("tilt_deg", 25.0, 40.0)):
        v = np.array([getattr(c, name) for c in cfgs])
        assert v.min() >= lo and v.max() <= hi and v.max() - v.min() > 0.8 * (hi - lo), name
    flagged = ensemble_flagged(cfgs)
    assert 0 < len(flagged) < len(cfgs)
    assert [c.n for c in ensemble_configs(256)] == n.tolist()          # seeded, repeatable
    sys, fun, pp = ensemble_state(cfgs[:3])
    assert sys.shape == (3,) and len(pp) == sum(c.n for c in cfgs[:3])
    assert np.all(sys["dt"] == sys["dt"][0]) and len(set(sys["mu_pp"].tolist())) == 3
