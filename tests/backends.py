"""numpy-in / numpy-out adapters over the oracle and over the GPU library,
so that the reference's test programs (tests/refcases.py) run against both."""
import numpy as np

from oracle import oracle as O


class OracleBackend:
    def __init__(self, prec):
        self.prec = prec

    def c2c(self, a, fmt, isign, inplace, skip):
        a = np.ascontiguousarray(a)
        return O.fft3d_c2c(a, fmt, isign, inplace=inplace, skip=skip, prec=self.prec)

    def r2c(self, x, fmt, skip):
        return O.fft3d_r2c(x, fmt, skip=skip, prec=self.prec)

    def c2r(self, c, nx, ny, nz, fmt, inplace, skip):
        return O.fft3d_c2r(np.ascontiguousarray(c), nx, ny, nz, fmt, inplace=inplace, skip=skip,
                           prec=self.prec)

    def transpose(self, kind, a):
        return O.transpose(a)


class GpuBackend:
    """Runs every call through the C ABI of libgbfft.so on cuda:0."""

    def __init__(self, prec):
        import gbfft
        self.g = gbfft
        self.prec = prec
        self.gprec = gbfft.PREC_DOUBLE if prec == "d" else gbfft.PREC_SINGLE
        self.engines = {}

    def engine(self, fmt, nx, ny, nz, inplace, skip):
        key = (fmt, nx, ny, nz, bool(inplace), tuple(bool(s) for s in skip) if skip else None)
        if key not in self.engines:
            self.engines[key] = self.g.Engine(fmt, nx, ny, nz, inplace=inplace, skip=skip,
                                              prec=self.gprec)
        return self.engines[key]

    def c2c(self, a, fmt, isign, inplace, skip):
        import torch
        nz, ny, nx = a.shape
        e = self.engine(fmt, nx, ny, nz, inplace, skip)
        x = torch.from_numpy(np.ascontiguousarray(a)).cuda()
        out = torch.empty_like(x)
        e.c2c(x, out, isign)
        torch.cuda.synchronize()
        return out.cpu().numpy()

    def r2c(self, x, fmt, skip):
        import torch
        nz, ny, nx = x.shape
        e = self.engine(fmt, nx, ny, nz, False, skip)
        xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
        out = e.empty_spectral()
        e.r2c(xd, out)
        torch.cuda.synchronize()
        return out.cpu().numpy()

    def c2r(self, c, nx, ny, nz, fmt, inplace, skip):
        import torch
        e = self.engine(fmt, nx, ny, nz, inplace, skip)
        cd = torch.from_numpy(np.ascontiguousarray(c)).cuda()
        out = e.empty_physical()
        e.c2r(cd, out)
        torch.cuda.synchronize()
        return out.cpu().numpy()

    def transpose(self, kind, a):
        import torch
        g = self.g
        kinds = {"x_to_y": g.X_TO_Y, "y_to_z": g.Y_TO_Z, "z_to_y": g.Z_TO_Y, "y_to_x": g.Y_TO_X}
        nz, ny, nx = a.shape
        is_c = np.iscomplexobj(a)
        prec = g.PREC_DOUBLE if a.dtype in (np.float64, np.complex128) else g.PREC_SINGLE
        src = torch.from_numpy(np.ascontiguousarray(a)).cuda()
        dst = torch.empty_like(src)
        g.transpose(kinds[kind], src, dst, nx, ny, nz, is_c, prec)
        torch.cuda.synchronize()
        return dst.cpu().numpy()

    def close(self):
        for e in self.engines.values():
            e.close()
        self.engines.clear()
