"""The Gaussian-process external potential (GaussianProcessPotential and
GPHeBenzenePotential, src/potential.cpp:244-392, 5586-5763) on the device.

Inputs are the reference's: a gp parameter file of "key = value" lines,
repeated keys giving the components of a vector (kernel.ell,
data.normOffset, data.normScale), and a binary training file whose rows are
four doubles x, y, z, (K^-1 Y) (potential.cpp:281-295).
"""
import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import PGB_FP64, dptr


def read_gp_params(path):
    """The parameter file as a dict; vector keys map to lists."""
    out = {}
    with open(path) as f:
        for line in f:
            line = line.split("#", 1)[0].strip()
            if not line or "=" not in line:
                continue
            k, v = (x.strip() for x in line.split("=", 1))
            out.setdefault(k, []).append(v)
    return {k: (v if len(v) > 1 else v[0]) for k, v in out.items()}


def read_training(path, n):
    """n rows of x, y, z, K^-1 Y (doubles, native byte order)."""
    data = np.fromfile(path, dtype=np.float64, count=4 * n)
    if data.size != 4 * n:
        raise ValueError("unexpected end of file while reading GP training data")
    return data.reshape(n, 4)


class GaussianProcess:
    """GaussianProcessPotential::GP over batches of positions."""

    def __init__(self, training, matern_nu, ell, norm_offset, norm_scale, standard_mean,
                 standard_std, mean, sigma2, side, periodic=(1, 1, 1), precision=PGB_FP64):
        self.lib = _lib.load()
        t = np.ascontiguousarray(training, dtype=np.float64).reshape(-1, 4)
        p = _lib.PgbGpParams()
        p.matern_nu = matern_nu
        for d in range(3):
            p.ell[d] = np.broadcast_to(ell, 3)[d]
            p.norm_offset[d] = np.broadcast_to(norm_offset, 3)[d]
            p.norm_scale[d] = np.broadcast_to(norm_scale, 3)[d]
            p.side[d] = np.broadcast_to(side, 3)[d]
            p.periodic[d] = int(np.broadcast_to(periodic, 3)[d])
        p.standard_mean, p.standard_std, p.mean, p.sigma2 = standard_mean, standard_std, mean, sigma2
        p.precision = precision
        h = C.c_void_p()
        rc = self.lib.pgb_gp_create(C.byref(p), dptr(t), len(t), C.byref(h))
        if rc != 0:
            raise _lib.PgbError(rc, (self.lib.pgb_gp_last_error(None) or b"").decode())
        self.h = h
        self.n = len(t)

    @classmethod
    def from_files(cls, param_file, side, periodic=(1, 1, 1), precision=PGB_FP64, base_dir=None):
        """The reference's gp parameter file and the training file it names."""
        g = read_gp_params(param_file)
        fv = lambda k: [float(x) for x in (g[k] if isinstance(g[k], list) else [g[k]])]
        if "matern" not in g["kernel.type"]:
            raise ValueError("only the matern kernel is supported")
        n = int(g["kernel.numTrainingPoints"])
        tf = g["kernel.trainingFileName"]
        if base_dir and not os.path.isabs(tf):
            tf = os.path.join(base_dir, tf)
        return cls(read_training(tf, n), fv("kernel.maternNu")[0], fv("kernel.ell"),
                   fv("data.normOffset"), fv("data.normScale"), float(g["data.standardMean"]),
                   float(g["data.standardStd"]), float(g["kernel.mean"]), float(g["kernel.sigma2"]),
                   side, periodic, precision)

    def _chk(self, rc):
        return _lib.check(rc, self.h, gp=True)

    def close(self):
        if getattr(self, "h", None):
            self.lib.pgb_gp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __call__(self, pos):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(pos))
        self._chk(self.lib.pgb_gp_eval(self.h, dptr(pos), dptr(out), len(pos)))
        return out

    def benzene(self, pos):
        """GPHeBenzenePotential::V over a batch of positions (K)."""
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(pos))
        self._chk(self.lib.pgb_gp_benzene_v(self.h, dptr(pos), dptr(out), len(pos)))
        return out

    def stream(self):
        return self.lib.pgb_gp_stream(self.h)
