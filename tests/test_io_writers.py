"""The library's trajectory writers against the reference's Python formatting (opendust.py:1071-1098):
every number as "{}".format writes a float, XYZ frames appended, CSV rows with csv.writer's line
ends. Host code only: these run without a GPU."""
import csv

import numpy as np

from opendust_gb300 import _lib


def _edge_values():
    v = [0.0, -0.0, 1.0, -1.0, 0.1, 1e-4, 9.999e-5, 1e-5, 1.5e-5, 1e15, 9.999999999999998e15, 1e16,
         1.5e16, 123456789012345.6, 1e22, 1e100, 1e-100, 5e-324, 2.2250738585072014e-308,
         1.7976931348623157e308, 1234567.8901234567, 0.30000000000000004, 2.0 ** 52, 2.0 ** 53 + 2,
         float("inf"), float("-inf"), float("nan")]
    return v


def test_format_double_matches_python_repr():
    rng = np.random.default_rng(0)
    mags = 10.0 ** rng.uniform(-12, 20, 20000)
    vals = list(mags * rng.choice([-1.0, 1.0], mags.size)) + _edge_values()
    # positions in nm of a simulation (lambda ~ 1e6 nm) and their float32 round trips
    pos = rng.uniform(-4e6, 4e6, 5000)
    vals += list(pos) + list(pos.astype(np.float32).astype(np.float64))
    bad = [(v, _lib.format_double(v), "{}".format(v)) for v in vals
           if _lib.format_double(v) != "{}".format(v)]
    assert not bad, bad[:5]


def _python_xyz(path, pos, frame):
    with open(path, "a") as f:
        f.write("{}\n{}\n".format(len(pos), frame))
        for x, y, z in pos:
            f.write("Ar\t{}\t{}\t{}\n".format(x, y, z))


def _python_csv(path, pos, density, mass):
    with open(path, "w") as f:
        w = csv.writer(f)
        w.writerow(["x", "y", "z", "density", "mass"])
        for x, y, z in pos:
            w.writerow([x, y, z, density, mass])


def test_xyz_and_csv_frames_byte_identical(tmp_path):
    rng = np.random.default_rng(1)
    pos = rng.uniform(-3.5e6, 3.5e6, (1000, 3))
    pos[0] = [0.0, -0.0, 1e-5]
    pos[1] = [1e16, -2.5e-7, 123.0]
    a, b = tmp_path / "lib.xyz", tmp_path / "py.xyz"
    for frame in range(3):
        _lib.write_xyz_frame(str(a), pos * (frame + 1), frame)
        _python_xyz(str(b), pos * (frame + 1), frame)
    assert a.read_bytes() == b.read_bytes()
    c, d = tmp_path / "lib0.csv", tmp_path / "py0.csv"
    _lib.write_csv_frame(str(c), pos, 1e14 * 1e-27, 1681.5124)
    _python_csv(str(d), pos, 1e14 * 1e-27, 1681.5124)
    assert c.read_bytes() == d.read_bytes()


def test_writer_reports_unwritable_path(tmp_path):
    import pytest
    with pytest.raises(_lib.OpenDustError) as e:
        _lib.write_xyz_frame(str(tmp_path / "no" / "such" / "dir.xyz"), np.zeros((2, 3)), 0)
    assert "dir.xyz" in str(e.value)


class _Recorder:
    def __init__(self, fail_at=None):
        self.frames, self.fail_at = [], fail_at

    def _write_frames(self, out, plasma, pos_nm, frame):
        if frame == self.fail_at:
            raise OSError(f"disk full at frame {frame}")
        self.frames.append((frame, float(pos_nm[0, 0])))


def test_frame_writer_keeps_order_and_reports_errors():
    import pytest

    from opendust_gb300.opendust import _FrameWriter
    rec = _Recorder()
    w = _FrameWriter(rec, None, None)
    for k in range(20):
        w.put(np.full((4, 3), float(k)), k)
    w.close()
    assert rec.frames == [(k, float(k)) for k in range(20)]
    rec = _Recorder(fail_at=3)
    w = _FrameWriter(rec, None, None)
    with pytest.raises(OSError, match="frame 3"):
        for k in range(50):
            w.put(np.zeros((4, 3)), k)
        w.close()
    with pytest.raises(OSError, match="frame 3"):  # close() joins the thread and re-raises
        w.close()
    assert not w._t.is_alive()
    assert [f for f, _ in rec.frames] == [0, 1, 2]


def test_restart_file_byte_identical_and_read_back(tmp_path):
    import pytest
    rng = np.random.default_rng(2)
    pos = rng.uniform(-3.5e6, 3.5e6, (3000, 3))
    vel = rng.normal(0, 0.3, (3000, 3))
    a, b = tmp_path / "lib.restart", tmp_path / "py.restart"
    _lib.write_restart_file(str(a), pos, vel)
    with open(b, "w") as f:  # the reference's loop (opendust.py:1109-1114)
        for j in range(3000):
            f.write("{}\t{}\t{}\t{}\t{}\t{}\n".format(pos[j, 0], pos[j, 1], pos[j, 2],
                                                      vel[j, 0], vel[j, 1], vel[j, 2]))
    assert a.read_bytes() == b.read_bytes()
    p2, v2 = _lib.read_restart_file(str(b), 3000)
    assert np.array_equal(p2, pos) and np.array_equal(v2, vel)  # shortest repr reads back exactly
    p3, _ = _lib.read_restart_file(str(b), 10)
    assert np.array_equal(p3, pos[:10])
    with pytest.raises(_lib.OpenDustError, match="fewer"):
        _lib.read_restart_file(str(b), 3001)
