"""Film output and image comparison without OpenEXR.

write_pfm / read_pfm follow the reference's PFM writer and reader
(core/imageio.cpp WriteImagePFM / ReadImagePFM): a "PF" header, the width and
height, the scale -1 (little-endian floats), then RGB floats row by row from
the top of the image, as ImageFilm::WriteImage passes them.

image_diff restates tools/exrdiff.cpp for RGB images: per channel value, the
relative difference |a - b| / a against the first image (values where both
are zero skipped), counts of differences above 0.5% ("small") and 5%
("big"), both images' averages and their relative delta, and the MSE over
3 * width * height values.  The images differ when tol == 0 and any small or
big difference exists, or when tol > 0 and 100 * |avg delta| exceeds tol.
(The reference reads RGBA and, as written, skips channel 0 -- red -- where it
means to skip alpha; here every colour channel is compared.)

    python -m pbrt_gb300.imageio a.pfm b.pfm [-d tol] [-o diff.pfm]
exits 1 when the images differ, like exrdiff.
"""
from __future__ import annotations

import sys

import numpy as np


def write_pfm(path: str, rgb) -> None:
    """rgb [yres, xres, 3] float32, row 0 at the top."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    if rgb.ndim != 3 or rgb.shape[2] != 3:
        raise ValueError("write_pfm: expected [yres, xres, 3]")
    h, w, _ = rgb.shape
    with open(path, "wb") as f:
        f.write(b"PF\n%d %d\n%f\n" % (w, h, -1.0))
        f.write(rgb.astype("<f4").tobytes())


def read_pfm(path: str) -> np.ndarray:
    """[yres, xres, 3] float32, row 0 at the top (the writer's order)."""
    data = open(path, "rb").read()
    parts = data.split(b"\n", 3)
    if parts[0].strip() != b"PF":
        raise ValueError(f"{path}: not a 3-channel PFM")
    w, h = (int(x) for x in parts[1].split())
    scale = float(parts[2])
    dt = "<f4" if scale < 0 else ">f4"
    return np.frombuffer(parts[3][: 12 * w * h], dtype=dt).astype(np.float32).reshape(h, w, 3)


def image_diff(a, b, tol: float = 0.0) -> dict:
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    if a.shape != b.shape:
        return {"differ": True, "reason": f"resolutions do not match: {a.shape} vs {b.shape}"}
    x = a.reshape(-1).astype(np.float64)
    y = b.reshape(-1).astype(np.float64)
    n = x.size
    keep = ~((x == 0) & (y == 0))
    xs, ys = x[keep], y[keep]
    with np.errstate(divide="ignore", invalid="ignore"):
        d = np.abs(xs - ys) / xs
    small = int(np.count_nonzero(d > 0.005))
    big = int(np.count_nonzero(d > 0.05))
    avg1, avg2 = float(xs.sum() / n), float(ys.sum() / n)
    lo = min(avg1, avg2)
    avg_delta = (avg1 - avg2) / lo if lo != 0 else (0.0 if avg1 == avg2 else float("inf"))
    mse = float(((xs - ys) ** 2).sum() / n)
    differ = (tol == 0.0 and (big > 0 or small > 0)) or (tol > 0.0 and 100.0 * abs(avg_delta) > tol)
    return {"differ": bool(differ), "big": big, "big_pct": 100.0 * big / n, "small": small,
            "small_pct": 100.0 * small / n, "avg1": avg1, "avg2": avg2, "avg_delta_pct": 100.0 * avg_delta,
            "mse": mse}


def main(argv=None) -> int:
    argv = list(sys.argv[1:] if argv is None else argv)
    tol, out, files = 0.0, None, []
    while argv:
        a = argv.pop(0)
        if a == "-d":
            tol = float(argv.pop(0))
        elif a == "-o":
            out = argv.pop(0)
        else:
            files.append(a)
    if len(files) != 2:
        print("usage: python -m pbrt_gb300.imageio [-d tol] [-o diff.pfm] image1.pfm image2.pfm")
        return 1
    a, b = read_pfm(files[0]), read_pfm(files[1])
    r = image_diff(a, b, tol)
    if r["differ"]:
        if "reason" in r:
            print(f"{files[0]}/{files[1]}:\n\t{r['reason']}")
            return 1
        print(f"{files[0]} {files[1]}\n\tImages differ: {r['big']} big ({r['big_pct']:.2f}%), "
              f"{r['small']} small ({r['small_pct']:.2f}%)\n\tavg 1 = {r['avg1']:g}, avg2 = {r['avg2']:g} "
              f"({r['avg_delta_pct']:f}% delta)\n\tMSE = {r['mse']:g}")
        if out:
            write_pfm(out, np.abs(a - b))
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
