"""File layouts of the reference's reconstruction programs.

GoldenC (origin/GoldenC/src/main.c):
  * phantom.dat  -- 512 x 512 numbers, whitespace separated, row-major
                    (read with fscanf "%lf", main.c:52-58)
  * I_result.txt / E_result.txt -- f and v written "%f " per value and a
                    newline per row (main.c:63-77; six decimals)

helical/rebin (helical/rebin/src/ms2d.cpp):
  * view table   -- one "pos,angle" line per projection, angle in degrees
                    (load_table, ms2d.cpp:30-62; pos is divided by 1000)
  * sinogram     -- NPROJ x NDETECTOR numbers, whitespace separated
                    (ms2d.cpp:270-275)

industry3d (industry3d/src/ct3d.cpp:199-214, testcase/shepp_logan.cpp:157-166):
  * .dr          -- a 1024-byte header (zeros when written by the generator)
                    followed by unsigned 16-bit samples [NPROJ][NDX][NDY]
"""
from __future__ import annotations

import numpy as np

GOLDNC_N = 512


def read_goldnc_image(path: str, n: int = GOLDNC_N) -> np.ndarray:
    """phantom.dat / I_result.txt / E_result.txt as an n x n float64 array."""
    with open(path) as fh:
        vals = np.array(fh.read().split(), dtype=np.float64)
    if vals.size < n * n:
        raise ValueError(f"{path}: {vals.size} values, need {n * n}")
    return vals[: n * n].reshape(n, n)


def write_goldnc_image(path: str, img: np.ndarray) -> None:
    """Writes like GoldenC's result files: "%f " per value, one row per line."""
    img = np.asarray(img, np.float64)
    with open(path, "w") as fh:
        for row in img:
            fh.write("".join("%f " % v for v in row))
            fh.write("\n")


def read_view_table(path: str):
    """helical/rebin view table: returns (pos_m, angle_deg) arrays."""
    pos, ang = [], []
    with open(path) as fh:
        for line in fh:
            line = line.strip()
            if not line:
                continue
            a, b = line.split(",")[:2]
            pos.append(float(a) / 1000.0)
            ang.append(float(b))
    return np.array(pos), np.array(ang)


def write_view_table(path: str, pos_mm, angle_deg) -> None:
    with open(path, "w") as fh:
        for p, a in zip(pos_mm, angle_deg):
            fh.write(f"{float(p)!r},{float(a)!r}\n")


def uniform_view_angles(angle_deg, tol: float = 1e-9):
    """(view0_deg, view_step_deg) of an evenly spaced angle table; raises when
    the table is not evenly spaced (the fan geometry holds a start and a step)."""
    a = np.asarray(angle_deg, np.float64)
    if a.size < 2:
        return float(a[0]) if a.size else 0.0, 0.0
    step = (a[-1] - a[0]) / (a.size - 1)
    if np.max(np.abs(a - (a[0] + step * np.arange(a.size)))) > tol * max(1.0, abs(step) * a.size):
        raise ValueError("view angles are not evenly spaced")
    return float(a[0]), float(step)


def read_text_sinogram(path: str, nproj: int, ndet: int) -> np.ndarray:
    with open(path) as fh:
        vals = np.array(fh.read().split(), dtype=np.float64)
    if vals.size < nproj * ndet:
        raise ValueError(f"{path}: {vals.size} values, need {nproj * ndet}")
    return vals[: nproj * ndet].reshape(nproj, ndet)


def write_text_sinogram(path: str, sino: np.ndarray) -> None:
    np.savetxt(path, np.asarray(sino, np.float64), fmt="%.17g")


DR_HEADER = 1024


def read_dr(path: str, nproj: int, ndx: int, ndy: int) -> np.ndarray:
    """industry3d .dr: skip 1024 header bytes, then uint16 [nproj][ndx][ndy]."""
    data = np.fromfile(path, dtype="<u2", offset=DR_HEADER, count=nproj * ndx * ndy)
    if data.size != nproj * ndx * ndy:
        raise ValueError(f"{path}: short file")
    return data.reshape(nproj, ndx, ndy)


def write_dr(path: str, samples: np.ndarray) -> None:
    s = np.ascontiguousarray(samples, dtype="<u2")
    with open(path, "wb") as fh:
        fh.write(bytes(DR_HEADER))
        fh.write(s.tobytes())


def counts_to_line_integrals(counts: np.ndarray, i0: float) -> np.ndarray:
    """-log(max(N, 1) / I0) as FP32, the sinogram the engine reconstructs."""
    return (-np.log(np.maximum(np.asarray(counts, np.float64), 1.0) / i0)).astype(np.float32)
