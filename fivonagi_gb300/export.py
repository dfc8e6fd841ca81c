"""Frame export in the reference's text formats, so its plot scripts read
the files unchanged, the taylor app's error measures, and images of the
headless display.

Formats (apps/hifu-beam/data_export.h:14-179,
apps/taylor-angle-xy/data_export.h:15-177):
  u1-NNNN.dat       whole-grid u1: header lines, a first row "NY y_0 ... y_NY-1",
                    then one row per x: "x u1(x, y_0) ... "; x = (i + MDX)/ISPF,
                    y = (j - MDY - NY/2)/ISPF (hifu)
  u1-cut-NNNN.dat   "x u1(x, y_cut)" along row JCUT
  u1max.dat         "x u1max(x, y_cut)" over lab columns 0 .. NX-1+MDX
  microphone_K.dat  "n T u1" per step, appended per frame with "## frame" and
                    "## T_final" lines
  u1-cfl.dat        "n T frame cfl std", std the running RMS of cfl - CFLWHISH
                    over frames (the first collected step is skipped)
  taylor: u1-cut-NNNN.dat "i x numeric analytic" along the oblique cut and
          u1-error.dat "frame T error_L1 error_L2 error_Li"

`Recorder` drives a run frame by frame (fv_run_until at DTPRINT spacing),
reading the device collection after each frame.
"""
from __future__ import annotations

import os

import numpy as np

from . import _abi
from .solver import Simulation

_f32 = np.float32


def _fmt(v) -> str:
    """Numbers as C++ ostream prints them by default (6 significant digits)."""
    return f"{float(v):.6g}"


def write_u1_grid(path: str, u1: np.ndarray, T: float, mdx: int, mdy: int, ispf: float) -> None:
    ny, nx = u1.shape
    ispf32 = float(_f32(ispf))
    with open(path, "w") as f:
        f.write(f"# T={float(T):.5g}\n")
        f.write("# Lines are parallel to y-axis, an columns parallel to x-axis.\n")
        f.write("# First line are y values, and first column x values.\n")
        f.write("# Left-top corner is the number of columns\n")
        ys = [(float(_f32(j - mdy - ny // 2)) / ispf32) for j in range(ny)]
        f.write(f"{ny} " + " ".join(_fmt(_f32(y)) for y in ys) + "  \n")
        for i in range(nx):
            x = _f32(float(_f32(i + mdx)) / ispf32)
            f.write(_fmt(x) + " " + " ".join(_fmt(v) for v in u1[:, i]) + " \n")


def write_u1_cut(path: str, u1: np.ndarray, T: float, mdx: int, ispf: float, ampl: float, jcut: int) -> None:
    ny, nx = u1.shape
    ispf32 = float(_f32(ispf))
    with open(path, "w") as f:
        f.write(f"# T={float(T):.5g}\n# AMPL={_fmt(_f32(ampl))}\n# x u1(x,y_cut)\n")
        for i in range(nx):
            x = _f32(float(_f32(i + mdx)) / ispf32)
            f.write(f"{_fmt(x)} {_fmt(u1[jcut, i])} \n")


def write_u1max(path: str, envelope: np.ndarray, mdx: int, nx: int, ispf: float, ampl: float) -> None:
    ispf32 = float(_f32(ispf))
    with open(path, "w") as f:
        f.write(f"# AMPL={_fmt(_f32(ampl))}\n# x u1max(x,y_cut)\n")
        for i in range(min(nx + mdx, len(envelope))):
            x = _f32(float(_f32(i)) / ispf32)
            f.write(f"{_fmt(x)} {_fmt(envelope[i])}\n")


def append_microphones(dirname: str, frame: int, n_first: int, T_final: float, T: np.ndarray,
                       probes: np.ndarray) -> None:
    for k in range(probes.shape[1]):
        path = os.path.join(dirname, f"microphone_{k + 1}.dat")
        with open(path, "w" if frame == 0 else "a") as f:
            if frame == 0:
                f.write("# n T u1\n")
            f.write(f"## frame = {frame}\n## T_final = {float(T_final):.5g}\n")
            for s in range(len(T)):
                f.write(f"{n_first + s + 1} {_fmt(T[s])} {_fmt(probes[s, k])}\n")


class CflLog:
    """u1-cfl.dat: one line per collected step, with the running RMS of
    cfl - CFLWHISH (summed over steps, divided by frames + 1, as the
    reference's export does); the first collected step of the run is
    skipped."""

    def __init__(self, path: str, cflwhish: float):
        self.path = path
        self.whish = float(_f32(cflwhish))
        self.acc = 0.0
        self.first = True

    def append(self, frame: int, n_first: int, T: np.ndarray, cfl: np.ndarray) -> None:
        with open(self.path, "w" if frame == 0 else "a") as f:
            if frame == 0:
                f.write("# n T frame cfl std\n")
                self.acc = 0.0
            for s in range(len(T)):
                if T[s] > 0:
                    if not self.first:
                        self.acc += (float(cfl[s]) - self.whish) ** 2
                        f.write(f"{n_first + s + 1} {_fmt(T[s])} {frame} {_fmt(cfl[s])} "
                                f"{_fmt(np.sqrt(self.acc / (frame + 1)))}\n")
                    self.first = False


def taylor_cut(u1: np.ndarray, p: _abi.FvParams, T: float, mdx: int, mdy: int):
    """The taylor app's oblique cut through the wave centre (apps/
    taylor-angle-xy/data_collect.h:37-96): u1 interpolated linearly between
    the two rows around the cut line, and the analytic tanh profile at the
    nearest row; returns (numeric, analytic) over the cut's columns. The
    reference computes this on the device at every step and keeps the last;
    here it is computed once per frame on the host, in FP32 with numpy's
    tan/tanh."""
    ny, nx = u1.shape
    f = _f32
    dx = f(f(p.xmax) / f(nx - 1))
    dy = f(f(p.ymax) / f(ny - 1))
    eta = f(f(nx) / f(p.xmax))
    th = f(p.angle)
    mdvx, mdvy, mdt = f(p.mdvx), f(p.mdvy), f(p.mdt)
    Tf = f(T)
    icenter = int(Tf * mdvx / dx) - mdx
    jcenter = ny // 2 + int((Tf - mdt) * mdvy / dy) - mdy
    half = int(f(5.0) * eta * f(np.cos(th)))
    rhoa, c = f(p.isp_rhoa), f(p.isp_c)
    num, ana = [], []
    for i in range(max(0, icenter - half), min(nx, icenter + half + 1)):
        ja = f(jcenter) + f(i - icenter) * (dx / dy) * f(np.tan(th))
        j0 = int(np.floor(ja))
        dj = f(j0 + 1) - ja
        if not (0 <= j0 and j0 + 1 < ny):
            continue
        num.append(float(dj * u1[j0, i] + (f(1) - dj) * u1[j0 + 1, i]))
        jj = int(np.floor(ja + f(0.5)))  # the row within half a cell of the cut
        arg = c * (f(i + mdx) * dx * f(np.cos(th)) + (f(jj + mdy - ny // 2) * dy + mdt * f(np.sin(th))) *
                   f(np.sin(th)) - Tf)
        ana.append(float(rhoa * f(np.tanh(arg))))
    return np.array(num), np.array(ana)


def error_norms(numeric: np.ndarray, analytic: np.ndarray):
    """Relative L1, L2 and L-infinity errors (taylor data_export.h:111-127)."""
    d = np.abs(analytic - numeric)
    a = np.abs(analytic)
    return (float(d.sum() / a.sum()), float(np.sqrt((d ** 2).sum() / (a ** 2).sum())), float(d.max() / a.max()))


class Recorder:
    """Runs a simulation frame by frame with device collection on, writing
    the reference's frame files into `outdir`. hifu-style apps record the
    four microphones at 0.5, 0.9, 1.0 and 1.1 ISPF on row JCUT and the
    central-peak envelope along that row (data_collect.h:51-102)."""

    def __init__(self, sim: Simulation, outdir: str, dtprint: float, jcut: int = 2):
        self.sim = sim
        self.p = sim.params
        self.outdir = outdir
        self.dtprint = float(dtprint)
        self.jcut = jcut
        self.frame = 0
        self.n_done = 0
        os.makedirs(outdir, exist_ok=True)
        ispf = _f32(self.p.isp_f)
        mics = [int(np.rint(ispf * _f32(0.5))), int(np.rint(ispf * _f32(0.9))), int(ispf),
                int(np.rint(ispf * _f32(1.1)))]
        self.taylor = self.p.app == _abi.FV_APP_TAYLOR_ANGLE_XY
        if self.taylor:
            sim.collect_enable(capacity=self.p.nx)
        else:
            sim.collect_enable(probes=[(m, jcut) for m in mics], envelope_row=jcut, envelope_len=4 * self.p.nx,
                               envelope_halfwidth=0.5)
        self.cfl = CflLog(os.path.join(outdir, "u1-cfl.dat"), self.p.cflwhish)

    def frame_step(self) -> dict:
        st = self.sim.calc_frame(self.dtprint)
        c = self.sim.collect_read()
        u1 = self.sim.get_state()[0]
        T, mdx, mdy = st["T"], st["mdx"], st["mdy"]
        tag = f"{self.frame:04d}"
        out = {"stats": st, "collected": c}
        if self.taylor:
            num, ana = taylor_cut(u1, self.p, T, mdx, mdy)
            with open(os.path.join(self.outdir, f"u1-cut-{tag}.dat"), "w") as f:
                f.write(f"# T={float(T):.5g}\n# i x numeric analytic\n")
                eta = _f32(_f32(self.p.nx) / _f32(self.p.xmax))
                for k in range(len(num)):
                    x = -5.0 + k / (float(eta) * np.cos(float(_f32(self.p.angle))))
                    f.write(f"{k} {_fmt(x)} {_fmt(num[k])} {_fmt(ana[k])}  \n")
            e = error_norms(num, ana) if len(num) else (float("nan"),) * 3
            with open(os.path.join(self.outdir, "u1-error.dat"), "w" if self.frame == 0 else "a") as f:
                if self.frame == 0:
                    f.write("# frame T error_L1 error_L2 error_Li\n")
                f.write(f"{self.frame} {float(T):.5g} {_fmt(e[0])} {_fmt(e[1])} {_fmt(e[2])}\n")
            out["errors"] = e
        else:
            write_u1_grid(os.path.join(self.outdir, f"u1-{tag}.dat"), u1, T, mdx, mdy, self.p.isp_f)
            write_u1_cut(os.path.join(self.outdir, f"u1-cut-{tag}.dat"), u1, T, mdx, self.p.isp_f, self.p.ampl,
                         self.jcut)
            write_u1max(os.path.join(self.outdir, "u1max.dat"), c["envelope"], mdx, self.p.nx, self.p.isp_f,
                        self.p.ampl)
            append_microphones(self.outdir, self.frame, self.n_done, T, c["T"], c["probes"])
        self.cfl.append(self.frame, self.n_done, c["T"], c["cfl"])
        self.n_done += c["steps"]
        self.frame += 1
        return out


def write_png(path: str, rgba: np.ndarray) -> None:
    """An RGBA8 image (rows, cols, 4) as a PNG file (zlib, no filtering)."""
    import struct
    import zlib

    rows, cols, _ = rgba.shape
    raw = b"".join(b"\x00" + rgba[r].astype(np.uint8).tobytes() for r in range(rows))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    ihdr = struct.pack(">IIBBBBB", cols, rows, 8, 6, 0, 0, 0)
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"IDAT", zlib.compress(raw, 6)) +
                chunk(b"IEND", b""))


def render_reference(u1: np.ndarray, ampl: float, plot_scale: float, width: int, height: int, zoom: int = 1,
                     i0: int = 0, j0: int = 0, jcut: int = -1) -> np.ndarray:
    """numpy restatement of fv_render without overlays (for tests): the
    map and cut-plot lightness, then the hue/lightness colour map."""
    ny, nx = u1.shape
    f = np.float32
    scale = f(1.0 / (plot_scale * ampl))
    rows = height + (128 if jcut >= 0 else 0)
    xs = np.arange(width)
    ii = np.clip(xs * zoom + i0, 0, nx - 1)
    light = np.zeros((rows, width), np.float32)
    for y in range(height):
        jj = min(max(y * zoom + j0, 0), ny - 1)
        light[y] = np.clip(u1[jj, ii] * scale * f(0.5) + f(0.5), 0, 1)
    if jcut >= 0:
        d = u1[jcut, ii] * scale * f(0.25)
        for yy in range(128):
            line = f(0.5) if yy == 64 else (f(0.25) if yy in (32, 96) else f(0))
            light[height + yy] = np.where(np.abs(f(yy) - f(64) - d * f(128)) < 1, f(1), line)
    hue = (180 + (f(360) * light).astype(np.int64)) % 360
    m2 = np.where(light <= 0.5, light * f(2), f(1))
    m1 = f(2) * light - m2

    def chan(h):
        h = ((h % 360) + 360) % 360
        v = np.where(h < 60, m1 + (m2 - m1) * h.astype(np.float32) / f(60),
                     np.where(h < 180, m2,
                              np.where(h < 240, m1 + (m2 - m1) * (240 - h).astype(np.float32) / f(60), m1)))
        return (f(255) * v).astype(np.uint8)

    out = np.empty((rows, width, 4), np.uint8)
    out[..., 0], out[..., 1], out[..., 2], out[..., 3] = chan(hue + 120), chan(hue), chan(hue - 120), 255
    return out
