"""dist_reader_gpu, the drop-in for ALMA's dist_reader (src/dist_reader.cpp):
it reads properties.msgpack.bin frames and writes the phonon distribution
of the listed boxes at the listed times.  Host code only: these tests build
frames with the library's own frame writer and check the four CSVs against
a numpy restatement of print_distribution (:270-508), to the 6 significant
digits the writer prints."""
import os
import subprocess

import numpy as np
import pytest

import btegpu
import pyoracle
import synth


def _case(tmp_path, times=(2.0, 3.0), ticks=40, boxes=(1, 3)):
    m = synth.mode_table(8, 3, 3, 300.0, config=100)
    g = synth.ribbon_geometry(200.0, 50.0, 5)
    synth.write_geometry_xml(str(tmp_path / "beam.xml"), g)
    synth.write_modes_file(str(tmp_path / "modes.bin"), m)
    spec = "".join(f'    <location bin="{b}"/>\n' for b in boxes)
    spec += "".join(f'    <time t="{t}"/>\n' for t in times)
    (tmp_path / "input.xml").write_text(
        '<beRTAMC2D>\n  <geometry file="beam.xml"/>\n  <time dt="1.0" maxtime="10"/>\n'
        f'  <material name="synthetic" database="modes.bin" thickness="{g["thickness"]!r}"/>\n'
        f'  <spectral>\n    <resolution ticks="{ticks}"/>\n{spec}  </spectral>\n</beRTAMC2D>\n')
    return m, g


def _frames(m, g, nframes=5, seed=3):
    rng = np.random.default_rng(seed)
    nbx, n = int(g["nboxes"]), m["omega"].size
    out, Hs = b"", []
    temps = list(np.asarray(g["Teq"], dtype=float))
    for f in range(nframes):
        H = np.zeros((nbx, n), dtype=np.int32)
        for b in range(nbx):
            if b == 2:
                continue  # an empty box: the (0, [42.0]) record
            k = rng.choice(np.arange(3, n), size=60, replace=False)
            H[b, k] = rng.integers(-40, 41, size=60)
        Hs.append(H)
        out += btegpu.debug_frame(float(f), 2e-23, temps, H)
    return out + b"0#", Hs, temps


def _areas(g):
    """Areas of the (convex, ordered) boxes by the shoelace formula."""
    out, off = [], 0
    for n in g["npoints"]:
        p = np.asarray(g["vertices"][2 * off:2 * (off + n)]).reshape(-1, 2)
        out.append(0.5 * abs(np.dot(p[:, 0], np.roll(p[:, 1], -1)) - np.dot(p[:, 1], np.roll(p[:, 0], -1))))
        off += n
    return out


def test_dist_reader_matches_restatement(built, tmp_path):
    m, g = _case(tmp_path)
    data, Hs, temps = _frames(m, g)
    (tmp_path / "properties.msgpack.bin").write_bytes(data)
    exe = os.path.join(os.path.dirname(built), "dist_reader_gpu")
    r = subprocess.run([exe, "input.xml", "properties.msgpack.bin"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    # the frames read back as written
    frames = btegpu.split_frames(data)
    t, E, T, hists = pyoracle.decode_berta_frame(frames[2])
    assert t == 2.0 and E == 2e-23 and T == temps
    assert hists[1] == {int(k): int(H) for k, H in enumerate(Hs[2][1]) if H != 0} and hists[2] == {}
    area = _areas(g)
    for b in (1, 3):
        d = np.loadtxt(tmp_path / f"deltaT_omega_{b}.csv", delimiter=",")
        jx = np.loadtxt(tmp_path / f"jx_omega_{b}.csv", delimiter=",")
        jy = np.loadtxt(tmp_path / f"jy_omega_{b}.csv", delimiter=",")
        fd_lines = (tmp_path / f"fd_{b}.csv").read_text().splitlines()
        assert d.shape == (3, 41) and d[0, 0] == -1.0       # mesh row, times 2 and 3
        assert fd_lines[0].startswith("# ") and fd_lines[1].startswith("# ") and len(fd_lines) == 4
        for row, frame in ((1, 2), (2, 3)):
            _, E, T, hists = pyoracle.decode_berta_frame(frames[frame])
            mesh, out = pyoracle.dist_reader_restated(m, area, g["thickness"], [1, 3], 40, hists, T, E)
            assert np.allclose(d[0, 1:], mesh, rtol=1e-5)
            assert d[row, 0] == frame
            dd, dx, dy, fd = out[b]
            for mine, ref in ((d[row, 1:], dd), (jx[row, 1:], dx), (jy[row, 1:], dy)):
                assert np.allclose(mine, ref, rtol=2e-5, atol=1e-5 * np.abs(ref).max())
            f = np.array(fd_lines[1 + row].split(","), dtype=float)
            assert f[0] == frame
            assert np.allclose(f[1:], fd, rtol=2e-5, atol=1e-5 * np.abs(fd).max())
    # it stopped at the last dump time and printed what the reference prints
    assert "*Read line 3" in r.stdout and "*Read line 4" not in r.stdout
    assert "Energy density of box 1 is" in r.stdout


def test_dist_reader_rejects_bad_input(built, tmp_path):
    m, g = _case(tmp_path, times=())
    (tmp_path / "properties.msgpack.bin").write_bytes(b"0#")
    exe = os.path.join(os.path.dirname(built), "dist_reader_gpu")
    r = subprocess.run([exe, "input.xml", "properties.msgpack.bin"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "time" in r.stderr
    r = subprocess.run([exe, "input.xml"], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "USAGE" in r.stdout
