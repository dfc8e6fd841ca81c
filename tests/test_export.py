"""Frame export formats (the reference's .dat layouts), error norms, PNG."""
import os

import numpy as np

from fivonagi_gb300 import export


def test_grid_and_cut_files_follow_the_reference_layout(tmp_path):
    ny, nx = 4, 5
    u1 = np.arange(ny * nx, dtype=np.float32).reshape(ny, nx) * np.float32(1e-3)
    g = os.path.join(tmp_path, "u1-0003.dat")
    export.write_u1_grid(g, u1, 1.25, 2, 0, 10.0)
    lines = open(g).read().splitlines()
    assert lines[0] == "# T=1.25" and lines[3].startswith("# Left-top")
    head = lines[4].split()
    assert head[0] == "4" and len(head) == 1 + ny and float(head[1]) == -0.2  # (0 - 0 - 2)/10
    row = lines[5].split()
    # six significant digits, as the reference's ofstream writes them
    assert float(row[0]) == 0.2 and np.allclose([float(v) for v in row[1:]], u1[:, 0], rtol=1e-5, atol=0)
    assert len(lines) == 5 + nx
    c = os.path.join(tmp_path, "u1-cut-0003.dat")
    export.write_u1_cut(c, u1, 1.25, 2, 10.0, 5e-3, 2)
    cl = open(c).read().splitlines()
    assert cl[:3] == ["# T=1.25", "# AMPL=0.005", "# x u1(x,y_cut)"]
    x, v = [float(t) for t in cl[3].split()]
    assert x == 0.2 and np.isclose(v, u1[2, 0], rtol=1e-5, atol=0)


def test_microphones_and_cfl_log_append_per_frame(tmp_path):
    d = str(tmp_path)
    T = np.array([0.1, 0.2], np.float32)
    pr = np.array([[1.0, 2.0], [3.0, 4.0]], np.float32)
    export.append_microphones(d, 0, 0, 0.2, T, pr)
    export.append_microphones(d, 1, 2, 0.4, T + np.float32(0.2), pr)
    m1 = open(os.path.join(d, "microphone_1.dat")).read().splitlines()
    assert m1[0] == "# n T u1" and m1[1] == "## frame = 0" and m1[3] == "1 0.1 1"
    assert "## frame = 1" in m1 and m1[-1] == "4 0.4 3"
    log = export.CflLog(os.path.join(d, "u1-cfl.dat"), 0.9)
    log.append(0, 0, np.array([0.1, 0.2], np.float32), np.array([0.9, 1.0], np.float32))
    cl = open(os.path.join(d, "u1-cfl.dat")).read().splitlines()
    # the first collected step is skipped; std = sqrt(sum (cfl - whish)^2 / (frame + 1))
    assert cl[0] == "# n T frame cfl std" and len(cl) == 2
    n, t, fr, cfl, std = cl[1].split()
    assert (n, fr) == ("2", "0") and abs(float(std) - abs(1.0 - float(np.float32(0.9)))) < 1e-6


def test_error_norms():
    a = np.array([1.0, -2.0, 3.0])
    n = np.array([1.5, -2.0, 2.0])
    l1, l2, li = export.error_norms(n, a)
    assert abs(l1 - 1.5 / 6.0) < 1e-15 and abs(l2 - np.sqrt(1.25 / 14.0)) < 1e-15 and abs(li - 1.0 / 3.0) < 1e-15


def test_png_writer_round_trip(tmp_path):
    import struct
    import zlib

    img = np.zeros((3, 4, 4), np.uint8)
    img[..., 0] = np.arange(12, dtype=np.uint8).reshape(3, 4) * 20
    img[..., 3] = 255
    path = tmp_path / "x.png"
    export.write_png(str(path), img)
    data = path.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    w, h = struct.unpack(">II", data[16:24])
    assert (w, h) == (4, 3)
    idat = data.index(b"IDAT")
    n = struct.unpack(">I", data[idat - 4:idat])[0]
    raw = zlib.decompress(data[idat + 4:idat + 4 + n])
    rows = [raw[r * 17 + 1:(r + 1) * 17] for r in range(3)]
    assert np.array_equal(np.frombuffer(b"".join(rows), np.uint8).reshape(3, 4, 4), img)


def test_render_reference_colour_map_extremes():
    u1 = np.array([[-1.0, 0.0, 1.0]], np.float32)
    img = export.render_reference(u1, ampl=1.0, plot_scale=1.0, width=3, height=1)
    # lightness 0 -> black, lightness 1 -> white
    assert tuple(img[0, 0, :3]) == (0, 0, 0) and tuple(img[0, 2, :3]) == (255, 255, 255)
    assert img[0, 1, 3] == 255
