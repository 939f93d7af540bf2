"""Observables and post-processing on the device: exact global mass and
momentum, the Strouhal number of a probe trace, the shear-wave viscosity fit,
and headless field export (reference-format .npy and colour-mapped PNG).

The reference does these on the host after each run: the probe FFT in
src/visualizations_utils.py:149-167, the decay fit in src/experiments.py:195-210,
PNG frames through PIL/matplotlib in src/experiments.py:638-647 and the
collective .npy writer save_mpiio in src/parallelization_utils.py:203-253.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np
import torch

from . import _arrays as A
from . import _lib


def mass_momentum(f) -> tuple:
    """(sum rho, sum jx, sum jy) of a reference-layout f[..., 9], exact: the sums
    are formed in 128-bit fixed point, independent of summation order."""
    ft = A.to_device(f)
    assert ft.shape[-1] == 9
    n = ft.numel() // 9
    lib = _lib.load()
    scratch = torch.empty(int(lib.lbm_reduce_scratch_bytes(n)), dtype=torch.uint8, device=ft.device)
    out = torch.empty(3, dtype=torch.float64, device=ft.device)
    _lib.call("lbm_reduce_moments_f64", ft.data_ptr(), n, scratch.data_ptr(), scratch.numel(), out.data_ptr(),
              A.stream())
    m, px, py = out.tolist()
    return m, px, py


def _as_trace(trace, device=None):
    if isinstance(trace, torch.Tensor):
        return trace.to(dtype=torch.float64, device=device or trace.device)
    return torch.as_tensor(np.asarray(trace, dtype=np.float64), device=device or "cpu")


def strouhal(trace, length: float, velocity: float, start: int = 0, method: str = "argmax",
             device=None) -> float:
    """St = f L / u of the dominant frequency f (cycles per time step) of trace[start:].

    method "argmax": f = |fftfreq[argmax |FFT(trace - mean)|]|, the reference's
    definition (visualizations_utils.py:157-167), resolved to one FFT bin
    (1 / len cycles per step).  method "interp": spectral_peak's sub-bin
    estimate.  Float64, on ``device`` (default: where the trace is; NumPy input
    on the host)."""
    t = _as_trace(trace, device)[start:]
    if method == "interp":
        return spectral_peak(t)[0] * length / velocity
    assert method == "argmax", "method is 'argmax' or 'interp'"
    spec = torch.fft.fft(t - t.mean()).abs()
    freq = torch.fft.fftfreq(t.numel(), 1.0, dtype=torch.float64, device=t.device)
    return float(freq[int(torch.argmax(spec))].abs()) * length / velocity


def spectral_peak(trace, start: int = 0, pad: int = 16, device=None) -> tuple:
    """Sub-bin frequency of the largest spectral peak of trace[start:], in cycles
    per sample: the mean is removed, a (symmetric) Hann window applied, the FFT
    zero-padded to ``pad`` times the length, and a Gaussian interpolation -- a
    parabola through the logarithms of the peak bin and its two neighbours --
    places the peak between bins (M. Gasior, J. L. Gonzalez, "Improving FFT
    frequency measurement resolution by parabolic and Gaussian spectrum
    interpolation", 2004).  Bins below 2 (unpadded) are left out,
    the remains of the mean.  Returns (frequency, bin, padded bin): the bin width
    1/len that the argmax estimate is quantised to, and 1/(pad len); the
    interpolation places the peak to a small fraction of the padded bin."""
    t = _as_trace(trace, device)[start:]
    n = t.numel()
    assert n >= 8, "trace too short"
    x = (t - t.mean()) * torch.hann_window(n, periodic=False, dtype=torch.float64, device=t.device)
    m = pad * n
    spec = torch.fft.rfft(x, n=m).abs()
    lo = 2 * pad
    k = lo + int(torch.argmax(spec[lo:]))
    k = min(k, spec.numel() - 2)
    a, b, c = torch.log(spec[k - 1:k + 2].clamp_min(1e-300)).tolist()
    den = a - 2.0 * b + c
    p = 0.5 * (a - c) / den if den != 0.0 else 0.0
    return (k + p) / m, 1.0 / n, 1.0 / m


def fit_decay_viscosity(amplitudes, times, eps: float, wavelength: float, iters: int = 50) -> float:
    """nu from amplitudes ~ eps exp(-nu k^2 t), k = 2 pi / wavelength, by Gauss-Newton
    least squares in float64 on the device (the fit of experiments.py:195-210)."""
    a = torch.as_tensor(amplitudes, dtype=torch.float64, device="cuda")
    t = torch.as_tensor(times, dtype=torch.float64, device="cuda")
    k2 = (2 * np.pi / wavelength) ** 2
    # start from the log-linear slope
    nu = float(-(torch.log(a.clamp_min(1e-300) / eps) * t).sum() / (k2 * (t * t).sum()))
    for _ in range(iters):
        model = eps * torch.exp(-nu * k2 * t)
        r = a - model
        jac = -k2 * t * model
        step = float((jac * r).sum() / (jac * jac).sum())
        nu -= step
        if abs(step) < 1e-15 * max(abs(nu), 1e-30):
            break
    return nu


# 256-entry colour map sampled from a smooth dark-blue -> green -> yellow ramp
def _colormap(n=256):
    x = np.linspace(0.0, 1.0, n)
    r = np.clip(0.27 + x * (-0.2 + x * 1.9) - x ** 3 * 0.97, 0, 1)
    g = np.clip(0.0 + x * 1.4 - x ** 2 * 0.5, 0, 1)
    b = np.clip(0.33 + x * (1.4 - x * 2.6) + x ** 3 * 1.0, 0, 1)
    return torch.tensor(np.stack([r, g, b], -1) * 255.0 + 0.5, dtype=torch.uint8)


def colour_frame(field: torch.Tensor) -> torch.Tensor:
    """(ny, nx, 3) uint8 image of a 2-D field f[x, y] normalised by its maximum, y up
    (the orientation of the reference's frames: cm.viridis(normalized.T))."""
    v = field.to(torch.float64)
    v = v / v.abs().max().clamp_min(1e-300)
    idx = (v.clamp(0, 1) * 255).round().to(torch.long)
    lut = _colormap().to(v.device)
    return lut[idx].transpose(0, 1).contiguous()


def write_png(path: str, rgb) -> None:
    """Minimal PNG writer (8-bit RGB, zlib), no imaging library needed."""
    img = rgb.cpu().numpy() if isinstance(rgb, torch.Tensor) else np.asarray(rgb)
    h, w, _ = img.shape
    raw = b"".join(b"\x00" + img[row].tobytes() for row in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(path, "wb") as fh:
        fh.write(b"\x89PNG\r\n\x1a\n")
        fh.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)))
        fh.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        fh.write(chunk(b"IEND", b""))


def save_velocity_frame(path: str, u) -> None:
    """|u| colour-mapped to a PNG file (the frames of experiments.py:638-647)."""
    ut = A.to_device(u)
    write_png(path, colour_frame(torch.linalg.norm(ut, dim=-1)))


def npy_bytes(arr: np.ndarray) -> bytes:
    """The .npy file save_mpiio (parallelization_utils.py:203-253) writes for a
    2-D array on one rank: format 1.0, the header dict padded with spaces so
    that magic + length + header end one byte short of a multiple of 16, then a
    newline, then the C-order data."""
    arr = np.ascontiguousarray(arr)
    assert arr.ndim == 2, "save_mpiio writes two-dimensional arrays"
    magic_str = b"\x93NUMPY\x01\x00"
    header = str({"descr": np.lib.format.dtype_to_descr(arr.dtype), "fortran_order": False,
                  "shape": (int(arr.shape[0]), int(arr.shape[1]))})
    while (len(header) + len(magic_str) + 2) % 16 != 15:
        header += " "
    header += "\n"
    return magic_str + np.int16(len(header)).astype("<i2").tobytes() + header.encode("latin-1") + arr.tobytes()


def save_field_npy(path: str, field) -> None:
    """A 2-D field (device tensor or host array) as the .npy file save_mpiio
    writes: the same bytes, readable with numpy.load."""
    if isinstance(field, torch.Tensor):
        field = field.detach().cpu().numpy()
    with open(path, "wb") as fh:
        fh.write(npy_bytes(np.asarray(field)))
