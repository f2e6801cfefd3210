"""af3d_avalanche, the reference's simulation program over the C ABI (csrc/af3d_avalanche.cpp):
its command line on the CPU, and on the GPU a short run (hopper filling, door, avalanche) whose
output files have the reference's shapes and whose final state is the one the same calls give
from Python, byte for byte."""
import os
import subprocess

import numpy as np
import pytest

DATAINPUT = """512         Number of particles.
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
"""


@pytest.fixture(scope="module")
def program():
    from avalancheflume3d_gb300 import build
    build.build()
    return build.PROGRAM


def test_command_line(program, tmp_path):
    r = subprocess.run([program, "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2 and "usage: af3d_avalanche" in r.stderr
    r = subprocess.run([program, "--input", str(tmp_path / "missing.dat")], capture_output=True, text=True)
    assert r.returncode == 1 and "missing.dat" in r.stderr
    # without --input the 16 lines come from standard input, as the reference reads them
    r = subprocess.run([program], input="".join(DATAINPUT.splitlines(True)[:9]), capture_output=True, text=True)
    assert r.returncode == 1 and "standard input" in r.stderr


@pytest.mark.gpu
def test_short_run_matches_the_same_calls_from_python(program, tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    (tmp_path / "DataInput.dat").write_text(DATAINPUT)
    fill, every, aval = 400, 200, 400
    r = subprocess.run([program, "--max-fill-steps", str(fill), "--out-every", str(every), "--t-end",
                        repr(aval * 1e-6 - 0.5e-6), "--checkpoint", "final.ckpt"],
                       cwd=tmp_path, input=DATAINPUT, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Opening hopper... Avalanche starts!" in r.stdout
    n = 512
    lines = lambda f: (tmp_path / f).read_text().splitlines()
    assert len(lines("mean_velocity_hst.csv")) == fill // every + aval // every
    assert len(lines("xcm_hst.csv")) == aval // every
    assert len(lines("snapshots_hst.xyz")) == (fill // every + aval // every) * (4 * n + 4)
    assert len(lines("last_config.dat")) == 4 + n
    # the same calls from Python
    v = af3d.load_datainput(str(tmp_path / "DataInput.dat"))
    sys, fun = af3d.derive_system(v)
    pp = af3d.generate_particles(sys)
    af3d.calculate_particle_parameters(pp)
    af3d.place_particles(sys, pp)
    af3d.set_initial_velocity(sys, pp)
    af3d.sphere_centres(pp)
    sys["tot_mass"] = float(np.sum(pp["mass"]))
    with af3d.Engine(sys, fun, ntags=int(v["ntags"]), phase=af3d.PHASE_FILL) as e:
        e.import_particles(pp)
        e.forces()
        e.swap_accel()
        e.step(fill)
        e.open_door()
        e.step(aval)
        want = e.export_particles()
    raw = np.fromfile(tmp_path / "final.ckpt", dtype=np.uint8)
    off = 64 + 256 + 24 + 168   # header, then the flume's system_par, Funnel, cell_par
    got = raw[off:off + 408 * n].view(af3d.PARTICLE)
    assert got.tobytes() == want[0].tobytes()
    acc = raw[off + 408 * n:off + 432 * n].view(np.float64).reshape(n, 3)
    assert acc.tobytes() == want[1].tobytes()


@pytest.mark.gpu
def test_resumed_run_continues_bit_for_bit(program, tmp_path):
    """A run stopped with --checkpoint and continued with --resume ends in the bytes of the run
    that did not stop."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    for d in ("straight", "first", "second"):
        (tmp_path / d).mkdir()
        (tmp_path / d / "DataInput.dat").write_text(DATAINPUT)
    run = lambda d, *a: subprocess.run([program, "--input", "DataInput.dat", *a], cwd=tmp_path / d,
                                       capture_output=True, text=True)
    r = run("straight", "--max-fill-steps", "200", "--out-every", "100", "--t-end", repr(400e-6 - 0.5e-6),
            "--checkpoint", "end.ckpt")
    assert r.returncode == 0, r.stderr
    r = run("first", "--max-fill-steps", "200", "--out-every", "100", "--t-end", repr(200e-6 - 0.5e-6),
            "--checkpoint", "mid.ckpt")
    assert r.returncode == 0, r.stderr
    r = run("second", "--resume", str(tmp_path / "first" / "mid.ckpt"), "--out-every", "100", "--t-end",
            repr(400e-6 - 0.5e-6), "--checkpoint", "end.ckpt")
    assert r.returncode == 0, r.stderr
    assert "Opening hopper" not in r.stdout   # the door was open already
    a = (tmp_path / "straight" / "end.ckpt").read_bytes()
    b = (tmp_path / "second" / "end.ckpt").read_bytes()
    assert a == b


def _csv_values(path):
    return np.array([[float(x) for x in line.replace(",", " ").split()] for line in
                     path.read_text().splitlines() if line.strip()])


@pytest.mark.gpu
def test_run_matches_the_oracle(program, tmp_path):
    """The drop-in program against the oracle driven through the reference's own sequence
    (avalanche_hst.cu:366-384 start-up pass, :401-601 hopper filling with the re-grid after every
    step whose counter is a multiple of 2000, :607-613 the door, :633-857 the avalanche) from the
    same DataInput.dat: the final state within the trajectory bar (1e-8 relative; exact FP64 mode,
    init_Verlet's sin/cos being the only operations not bit-identical) and every value of
    mean_velocity_hst.csv and xcm_hst.csv equal to the six decimals they are printed with (%lf),
    up to one unit in the last place where the two runs' values straddle a rounding boundary."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    from oracle.pyoracle import PHASE_AVALANCHE, PHASE_FILL, Oracle, OracleRun, xfinal
    fill, every, aval = 100, 50, 100
    run_dir, orc_dir = tmp_path / "program", tmp_path / "oracle"
    run_dir.mkdir()
    orc_dir.mkdir()
    r = subprocess.run([program, "--max-fill-steps", str(fill), "--out-every", str(every), "--t-end",
                        repr(aval * 1e-6 - 0.5e-6), "--checkpoint", "final.ckpt"],
                       cwd=run_dir, input=DATAINPUT, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    # the oracle from the same input, the reference's initial state and call sequence
    (orc_dir / "DataInput.dat").write_text(DATAINPUT)
    v = af3d.load_datainput(str(orc_dir / "DataInput.dat"))
    sys, fun = af3d.derive_system(v)
    pp = af3d.generate_particles(sys)
    af3d.calculate_particle_parameters(pp)
    af3d.place_particles(sys, pp)
    af3d.set_initial_velocity(sys, pp)
    af3d.sphere_centres(pp)
    sys["tot_mass"] = float(np.sum(pp["mass"]))
    run = OracleRun(Oracle(), sys, fun, pp, ntags=int(v["ntags"]))
    assert run.seed_accel(PHASE_FILL) == 0
    vm, xc = str(orc_dir / "mean_velocity_hst.csv"), str(orc_dir / "xcm_hst.csv")
    cc = 0
    while cc < fill:
        assert run.step(every, PHASE_FILL, cc0=cc) == 0
        cc += every
        af3d.append_snapshot(run.pp, run.sys, PHASE_FILL, vmean=vm, xcm=xc)
    run.sys["side"][0] = xfinal(run.sys)
    run.sys["time"] = 0.0
    cc = 0
    while cc < aval:
        assert run.step(every, PHASE_AVALANCHE, cc0=cc) == 0
        cc += every
        af3d.append_snapshot(run.pp, run.sys, PHASE_AVALANCHE, vmean=vm, xcm=xc)
    n = int(v["npart"])
    raw = np.fromfile(run_dir / "final.ckpt", dtype=np.uint8)
    off = 64 + 256 + 24 + 168
    got = raw[off:off + 408 * n].view(af3d.PARTICLE)
    for f in ("rr", "vv", "ww", "Rmatx", "Rmaty", "Rmatz", "rr_s"):
        scale = max(1.0, float(np.max(np.abs(run.pp[f]))))
        err = float(np.max(np.abs(got[f] - run.pp[f]))) / scale
        assert err <= 1e-8, "%s: max rel error %.3e" % (f, err)
    for name in ("mean_velocity_hst.csv", "xcm_hst.csv"):
        a, b = _csv_values(run_dir / name), _csv_values(orc_dir / name)
        assert a.shape == b.shape and a.size > 0, (name, a.shape, b.shape)
        err = np.max(np.abs(a - b) - 1e-8 * np.abs(b))
        assert err <= 1.0000001e-6, "%s: values differ by %.3e beyond the printed precision" % (name, err)
