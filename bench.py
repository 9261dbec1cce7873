#!/usr/bin/env python
"""Benchmark of the GB300 3D FFT backend on its headline workload.

Default workload: 3D r2c forward then c2r backward on a 1024 x 1024 x 512
real FP32 grid (PHYSICAL_IN_X), one step = one round trip.  The metric is
GPts/s = nx*ny*nz / t(r2c + c2r), summed over ranks (each rank runs its own
grid: replicas, no data-path collective).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
  python bench.py --impl reference ...   (the reference's CPU path)

`value` is measured with the input already resident in HBM (CUDA events on
the launching stream, K steps between a barrier + synchronize on both
sides, max over ranks).  `e2e` is the same metric through the C ABI with
host buffers: every step copies the input from pinned host memory, runs
r2c + c2r, and copies the result back.  Inputs (2 GiB real + 2.1 GiB
spectral) are larger than the 129 MB L2, so no flush is needed between
steps.  The CPU leg times whole round trips of the oracle -- the restated
generic backend of the reference -- on all host cores, and scipy.fft
(pocketfft) beside it.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "2decomp-fft_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "3D r2c+c2r GPts/s & %HBM roofline; split-TC vs plain FP32 at rel-L2≤1e-6"

WORKLOADS = {
    # name: (nx, ny, nz, format, precision, input kind)
    "r2c_c2r_1024x1024x512_f32_x": (1024, 1024, 512, 1, 4, "gauss_modes"),
    "r2c_c2r_1024x1024x512_f32_z": (1024, 1024, 512, 3, 4, "gauss_modes"),
    "r2c_c2r_64x64x64_f64_x": (64, 64, 64, 1, 8, "uniform"),
    "r2c_c2r_384x400x243_f64_x": (384, 400, 243, 1, 8, "uniform"),
    "r2c_c2r_384x400x243_f32_x": (384, 400, 243, 1, 4, "uniform"),
    "r2c_c2r_360x270x210_f64_x": (360, 270, 210, 1, 8, "uniform"),
    "r2c_c2r_360x270x210_f32_x": (360, 270, 210, 1, 4, "uniform"),
    "r2c_c2r_256x256x256_f32_x": (256, 256, 256, 1, 4, "uniform"),
    # profiling sizes: the x/y lines of the 1024x1024x512 grid at ~1/4 the memory,
    # its 512-point z lines (flat planes of 257-value rows) at ~1/8
    "r2c_c2r_1024x1024x128_f32_x": (1024, 1024, 128, 1, 4, "gauss_modes"),
    "r2c_c2r_512x256x512_f32_x": (512, 256, 512, 1, 4, "gauss_modes"),
    "r2c_c2r_1024x64x512_f32_x": (1024, 64, 512, 1, 4, "gauss_modes"),
    # the PHYSICAL_IN_Z grid's 512-point strided real lines at 1/8 the memory
    "r2c_c2r_512x256x512_f32_z": (512, 256, 512, 3, 4, "gauss_modes"),
    # axis lengths off the fast paths: the largest prime one shared-memory tile
    # takes (a direct-sum stage), a power of two beyond one tile (one radix
    # stage per kernel through scratch), a prime beyond one tile (a global
    # direct sum accumulated in double)
    "r2c_c2r_8191x64x64_f32_x": (8191, 64, 64, 1, 4, "uniform"),
    "r2c_c2r_65536x32x32_f32_x": (65536, 32, 32, 1, 4, "uniform"),
    "r2c_c2r_16411x16x16_f64_x": (16411, 16, 16, 1, 8, "uniform"),
}
DEFAULT_WORKLOAD = "r2c_c2r_1024x1024x512_f32_x"
BATCH_WORKLOAD = "batched_64_grids_f32"
# real-to-real (DCT-II on every axis, default windows: the last point of each
# axis left out) forward + backward: name -> (nx, ny, nz, precision, kinds)
# transposes plus c2c: the x -> y -> z -> y -> x transpose chain on a 256^3
# real64 and complex128 array (at one rank each transpose is an identity
# copy, bit for bit), then a 3D c2c forward + backward in complex64
C2C_WORKLOAD = "c2c_transposes_256x256x256"
DTT_WORKLOADS = {
    "r2r_dct2_256x256x256_f64_x": (256, 256, 256, 8, (2, 2, 2)),
    "r2r_dct2_256x256x256_f32_x": (256, 256, 256, 4, (2, 2, 2)),
    # 257-point axes: 256-point windows, 512-point extensions
    "r2r_dct2_257x257x257_f32_x": (257, 257, 257, 4, (2, 2, 2)),
    "r2r_dct2_257x257x257_f64_x": (257, 257, 257, 8, (2, 2, 2)),
}


# ---------------------------------------------------------------------------
# ranks
# ---------------------------------------------------------------------------
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _dist():
    try:
        import torch.distributed as dist
        return dist if dist.is_available() and dist.is_initialized() else None
    except Exception:
        return None


def barrier():
    d = _dist()
    if d is not None:
        d.barrier()


def max_over_ranks(x):
    """Largest value of x over all ranks (the step time the job sees)."""
    d = _dist()
    if d is None:
        return float(x)
    import torch
    dev = "cuda" if d.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x):
    d = _dist()
    if d is None:
        return float(x)
    import torch
    dev = "cuda" if d.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    d.all_reduce(t, op=d.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            if self.t:
                self.t.join(timeout=2)

    def summary(self, t0, t1):
        rows = []
        for ts, line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            rows.append((ts, parts))
        inside = [r for r in rows if t0 - 0.15 <= r[0] <= t1 + 0.15] or rows
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}

        def num(v):
            try:
                return float(v)
            except Exception:
                return None

        sm = sorted(x for x in (num(p[1]) for _, p in inside) if x is not None)
        smax = max((x for x in (num(p[2]) for _, p in inside) if x is not None), default=None)
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, p in inside:
            for name, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        pw = [x for x in (num(p[3]) for _, p in inside) if x is not None]
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(inside),
                "power_w_max": max(pw) if pw else None}


# ---------------------------------------------------------------------------
# host side of the end-to-end leg
# ---------------------------------------------------------------------------
def gpu_local_cpus(dev_index):
    """CPUs of the GPU's NUMA node (sysfs local_cpulist of its PCI device),
    restricted to this process's affinity; empty when unknown."""
    import torch
    try:
        p = torch.cuda.get_device_properties(dev_index)
        bus = "%04x:%02x:%02x.0" % (p.pci_domain_id, p.pci_bus_id, p.pci_device_id)
        text = open("/sys/bus/pci/devices/%s/local_cpulist" % bus).read().strip()
    except Exception:
        return set()
    cpus = set()
    for part in text.split(","):
        part = part.strip()
        if "-" in part:
            a, b = part.split("-")
            cpus |= set(range(int(a), int(b) + 1))
        elif part:
            cpus.add(int(part))
    return cpus & set(os.sched_getaffinity(0))


def bind_near_gpu(dev_index):
    """Run this process on the GPU's NUMA node, so that pinned host buffers
    allocated afterwards sit next to the GPU.  Returns the CPU list used."""
    cpus = gpu_local_cpus(dev_index)
    if cpus and cpus != set(os.sched_getaffinity(0)):
        try:
            os.sched_setaffinity(0, cpus)
        except Exception:
            pass
    return sorted(os.sched_getaffinity(0))


# syscall numbers of the memory-policy calls (Linux generic table on arm64)
_SYSCALLS = {"aarch64": {"set_mempolicy": 237, "move_pages": 239},
             "x86_64": {"set_mempolicy": 238, "move_pages": 279}}
_MPOL_DEFAULT, _MPOL_BIND = 0, 2


def gpu_numa_node(dev_index):
    """NUMA node of the GPU's PCI device (sysfs numa_node), -1 when unknown."""
    import torch
    try:
        p = torch.cuda.get_device_properties(dev_index)
        bus = "%04x:%02x:%02x.0" % (p.pci_domain_id, p.pci_bus_id, p.pci_device_id)
        return int(open("/sys/bus/pci/devices/%s/numa_node" % bus).read().strip())
    except Exception:
        return -1


def _syscall(name, *args):
    import ctypes
    import platform
    nr = _SYSCALLS.get(platform.machine(), {}).get(name)
    if nr is None:
        return -1
    libc = ctypes.CDLL(None, use_errno=True)
    libc.syscall.restype = ctypes.c_long
    return libc.syscall(ctypes.c_long(nr), *args)


def fault_in_on_node(addr, nbytes, node):
    """Touch every page of [addr, addr + nbytes) with this thread's memory
    policy bound to `node`, so that the pages are allocated there (the
    default policy falls back to the far node when the near one is full of
    page cache).  Returns False when the binding could not be set."""
    import ctypes
    mask = (ctypes.c_ulong * 16)()
    mask[node // 64] |= 1 << (node % 64)
    if _syscall("set_mempolicy", ctypes.c_int(_MPOL_BIND), mask, ctypes.c_ulong(16 * 64)) != 0:
        return False
    try:
        ctypes.memset(addr, 0, nbytes)
    finally:
        _syscall("set_mempolicy", ctypes.c_int(_MPOL_DEFAULT), None, ctypes.c_ulong(0))
    return True


def fraction_on_node(addr, nbytes, node, samples=64):
    """Share of `samples` pages spread over the range that sit on `node`
    (move_pages with no target nodes reports each page's node)."""
    import ctypes
    page = os.sysconf("SC_PAGESIZE")
    npages = max(1, nbytes // page)
    k = min(samples, npages)
    pages = (ctypes.c_void_p * k)(*[addr + (i * npages // k) * page for i in range(k)])
    status = (ctypes.c_int * k)()
    if _syscall("move_pages", ctypes.c_int(0), ctypes.c_ulong(k), pages, None, status, ctypes.c_int(0)) != 0:
        return None
    return round(sum(1 for v in status if v == node) / k, 3)


class HostBuffers:
    """Pinned host buffers of the end-to-end leg, on the GPU's NUMA node: an
    anonymous mapping whose pages are faulted in under a memory binding to
    the node, then page-locked in place (cudaHostRegister).  The default
    pinned allocator takes pages wherever the kernel finds room, which after
    other work on the machine can be the far node, at about half the host
    link's bandwidth.  Falls back to the default allocator when the node is
    unknown or a call fails, and says so in `placement()`."""

    def __init__(self, dev_index):
        self.node = gpu_numa_node(dev_index)
        self.keep = []      # (mmap, address, bytes) of registered buffers
        self.fallback = None
        self.share = []

    def empty(self, shape, dtype):
        import ctypes
        import mmap
        import torch
        numel = 1
        for d in shape:
            numel *= int(d)
        nbytes = numel * torch.empty((), dtype=dtype).element_size()
        if self.node >= 0 and self.fallback is None:
            try:
                mm = mmap.mmap(-1, nbytes)
                addr = ctypes.addressof(ctypes.c_char.from_buffer(mm))
                if not fault_in_on_node(addr, nbytes, self.node):
                    raise OSError("set_mempolicy failed")
                err = torch.cuda.cudart().cudaHostRegister(addr, nbytes, 0)
                if int(err) != 0:
                    raise OSError("cudaHostRegister: %s" % err)
                self.keep.append((mm, addr, nbytes))
                frac = fraction_on_node(addr, nbytes, self.node)
                if frac is not None:
                    self.share.append(frac)
                return torch.frombuffer(mm, dtype=dtype, count=numel).view(shape)
            except Exception as exc:  # noqa: BLE001
                self.fallback = str(exc)
        return torch.empty(shape, dtype=dtype, pin_memory=True)

    def placement(self):
        if self.node < 0:
            return {"numa_node": None, "how": "default pinned allocator (the GPU's node is unknown)"}
        if self.fallback:
            return {"numa_node": self.node, "how": "default pinned allocator (%s)" % self.fallback}
        return {"numa_node": self.node, "share_of_pages_on_node": min(self.share) if self.share else None,
                "how": "pages faulted in under set_mempolicy(MPOL_BIND) to the GPU's node, then cudaHostRegister"}

    def release(self):
        import torch
        torch.cuda.synchronize()
        for mm, addr, _ in self.keep:
            torch.cuda.cudart().cudaHostUnregister(addr)
        self.keep = []


def link_gbs(host, dev, stream, reps=3, host2=None):
    """Host-link bandwidth seen by this process: host->device, device->host
    and both at once (each direction), GB/s, copies of `host` (pinned) to
    and from `dev` timed with CUDA events.  `host` keeps its values (the
    device->host leg writes back what the host->device leg copied); the
    concurrent leg overwrites `host2`, a pinned buffer of `host`'s shape."""
    import torch
    nb = host.numel() * host.element_size()
    other = torch.cuda.Stream(dev.device)
    dev2 = torch.empty_like(dev)
    if host2 is None:
        host2 = torch.empty_like(host, pin_memory=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    for name, fn in (("h2d", lambda: dev.copy_(host, non_blocking=True)),
                     ("d2h", lambda: host.copy_(dev, non_blocking=True))):
        with torch.cuda.stream(stream):
            fn()
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
        torch.cuda.synchronize()
        out[name] = round(reps * nb / (e0.elapsed_time(e1) * 1e-3) / 1e9, 1)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(reps):
        with torch.cuda.stream(stream):
            dev.copy_(host, non_blocking=True)
        with torch.cuda.stream(other):
            host2.copy_(dev2, non_blocking=True)
    torch.cuda.synchronize()
    out["both_each"] = round(reps * nb / (time.perf_counter() - t) / 1e9, 1)
    return out


# ---------------------------------------------------------------------------
# inputs
# ---------------------------------------------------------------------------
def make_input(nx, ny, nz, kind, dtype, device):
    """Seeded synthetic field of the workload's shape (nz, ny, nx)."""
    import torch
    if kind == "gauss_modes":
        # N(0, 1) noise (seed 3) plus 8 modes 10 sin(2 pi (kx x/nx + ky y/ny
        # + kz z/nz) + phi), k uniform in 1..8 per axis, phi uniform (seed 4)
        g = torch.Generator(device=device).manual_seed(3)
        x = torch.randn((nz, ny, nx), generator=g, device=device, dtype=torch.float32)
        import numpy as np
        rng = np.random.default_rng(4)
        xs = torch.arange(nx, device=device, dtype=torch.float64) / nx
        ys = torch.arange(ny, device=device, dtype=torch.float64) / ny
        zs = torch.arange(nz, device=device, dtype=torch.float64) / nz
        for _ in range(8):
            kx, ky, kz = (int(v) for v in rng.integers(1, 9, size=3))
            phi = float(rng.uniform(0, 2 * np.pi))
            arg = (2 * np.pi * (kx * xs[None, None, :] + ky * ys[None, :, None] + kz * zs[:, None, None]) + phi)
            x += (10.0 * torch.sin(arg)).to(torch.float32)
        return x.to(dtype).contiguous()
    g = torch.Generator(device=device).manual_seed(5)
    return (torch.rand((nz, ny, nx), generator=g, device=device, dtype=torch.float64) * 2 - 1).to(dtype)


# ---------------------------------------------------------------------------
# CPU baseline: whole round trips of the oracle (and of pocketfft) on the host
# ---------------------------------------------------------------------------
def host_input(nx, ny, nz, prec, seed=3):
    """Seeded N(0, 1) host field of the workload's shape; the cost of a line
    FFT does not depend on the values."""
    import numpy as np
    rt = np.float32 if prec == 4 else np.float64
    return np.random.default_rng(seed).standard_normal((nz, ny, nx), dtype=rt)


def cpu_round_trips(x, fmt, prec, steps, warmup, threads=None):
    """Time whole r2c + c2r round trips of the oracle -- the restated generic
    backend, every line of all six passes -- as the reference's own test
    programs time them (examples/fft_physical_x/fft_r2c_x.f90:77-128: one
    untimed warm-up round trip, then the mean of ntest timed ones).  The
    arrays are allocated once and the oracle's work arrays persist across
    calls, as the reference's decomp_pool buffers do.  Returns (seconds per
    round trip, threads)."""
    import numpy as np
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    O.set_threads(threads)
    p = "d" if prec == 8 else "s"
    nz, ny, nx = x.shape
    ct = np.complex64 if prec == 4 else np.complex128
    spec = np.empty(O.spectral_shape(nx, ny, nz, fmt), dtype=ct)
    y = np.empty_like(x)
    for _ in range(warmup):
        O.fft3d_r2c_into(x, spec, fmt, p)
        O.fft3d_c2r_into(spec, y, fmt, p)
    times = []
    for _ in range(steps):
        t = time.perf_counter()
        O.fft3d_r2c_into(x, spec, fmt, p)
        O.fft3d_c2r_into(spec, y, fmt, p)
        times.append(time.perf_counter() - t)
    O.pool_release()
    return sum(times) / len(times), threads


def scipy_round_trips(x, fmt, steps, warmup, threads=None):
    """The FFTW-class CPU stand-in: scipy.fft (pocketfft) rfftn + irfftn in
    the input's precision with `workers` threads, timed like
    cpu_round_trips.  Returns (seconds per round trip, threads, version) or
    None when scipy is missing."""
    try:
        import scipy
        import scipy.fft as sfft
    except Exception:
        return None
    threads = threads or os.cpu_count() or 1
    nz, ny, nx = x.shape
    axes = (0, 1, 2) if fmt == 1 else (2, 1, 0)
    shape = (nz, ny, nx) if fmt == 1 else (nx, ny, nz)

    def rt():
        s = sfft.rfftn(x, axes=axes, workers=threads)
        return sfft.irfftn(s, s=shape, axes=axes, workers=threads)

    for _ in range(warmup):
        rt()
    times = []
    for _ in range(steps):
        t = time.perf_counter()
        rt()
        times.append(time.perf_counter() - t)
    return sum(times) / len(times), threads, scipy.__version__


def cpu_baseline(nx, ny, nz, fmt, prec, steps=2, warmup=1, x=None):
    """The cpu_baseline object of the GPU arm's line: the oracle's whole
    round trips (the value) and scipy.fft's beside it."""
    x = host_input(nx, ny, nz, prec) if x is None else x
    npts = nx * ny * nz
    sec, thr = cpu_round_trips(x, fmt, prec, steps, warmup)
    out = {"value": round(npts / sec / 1e9, 5), "unit": "GPts/s", "cores": thr, "kind": "port",
           "ms_per_round_trip": round(sec * 1e3, 1),
           "sample": "oracle (restated generic backend, Glassman FFT, %s build), OpenMP over lines on %d "
                     "host threads: whole r2c+c2r round trips of the full grid (every line of all 6 passes), "
                     "%d untimed warm-up then the mean of %d" % ("double" if prec == 8 else "single", thr,
                                                                 warmup, steps)}
    sp = scipy_round_trips(x, fmt, steps, warmup)
    if sp is not None:
        out["scipy_fft"] = {"value": round(npts / sp[0] / 1e9, 5), "unit": "GPts/s", "cores": sp[1],
                            "ms_per_round_trip": round(sp[0] * 1e3, 1),
                            "sample": "scipy %s scipy.fft.rfftn + irfftn (pocketfft, %s, workers=%d), "
                                      "%d warm-up then the mean of %d whole round trips"
                                      % (sp[2], "float32" if prec == 4 else "float64", sp[1], warmup, steps)}
    return out


# ---------------------------------------------------------------------------
# accuracy against FP64
# ---------------------------------------------------------------------------
def fp64_accuracy(x_dev, spec_dev, fmt):
    import numpy as np
    try:
        import scipy.fft as sfft
        kw = {"workers": os.cpu_count() or 1}
    except Exception:
        sfft, kw = np.fft, {}
    x = x_dev.cpu().numpy().astype(np.float64)
    if fmt == 1:
        ref = sfft.rfftn(x, axes=(0, 1, 2), **kw)
    else:
        ref = sfft.rfftn(x, axes=(2, 1, 0), **kw)
    got = spec_dev.cpu().numpy()
    d = got.astype(np.complex128) - ref
    rel = float(np.linalg.norm(d) / np.linalg.norm(ref))
    mx = float(np.abs(d).max() / np.abs(ref).max())
    return rel, mx


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------
def run_gb300(args):
    import torch
    import gbfft
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    cpus = bind_near_gpu(local)
    nx, ny, nz, fmt, prec, kind = WORKLOADS[args.workload]
    rdt = torch.float32 if prec == 4 else torch.float64
    gbfft.lib()

    form = {"split": gbfft.FORM_SPLIT, "split_tc": gbfft.FORM_SPLIT_TC}.get(args.form, gbfft.FORM_PLAIN)
    eng = gbfft.Engine(fmt, nx, ny, nz, prec=prec, form=form)
    x = make_input(nx, ny, nz, kind, rdt, dev)
    spec = eng.empty_spectral(device=dev)
    y = torch.empty_like(x)
    stream = torch.cuda.current_stream(dev)
    npts = nx * ny * nz

    def step():
        eng.r2c(x, spec, stream)
        eng.c2r(spec, y, stream)

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    l0 = gbfft.launch_count()
    t_wall0 = time.time()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    t_wall1 = time.time()
    barrier()
    launches = gbfft.launch_count() - l0
    ms = e0.elapsed_time(e1) / args.steps
    ms_max = max_over_ranks(ms)
    total_pts = sum_over_ranks(npts)
    value = total_pts / (ms_max * 1e-3) / 1e9

    # per-pass device times (events around each pass on the same stream)
    eng.set_profiling(True)
    prof_steps = max(3, min(args.steps, 10))
    for _ in range(prof_steps):
        step()
    torch.cuda.synchronize()
    prof = eng.profile()
    eng.set_profiling(False)
    clocks.stop()
    clk = clocks.summary(t_wall0, t_wall1)

    passes = {}
    for name, (n, tms, by) in prof.items():
        passes[name] = {"launches_per_step": n / prof_steps, "ms_per_launch": tms / n,
                        "gbs": by / (tms * 1e-3) / 1e9, "bytes_per_launch": by / n}
    dom = max(prof.items(), key=lambda kv: kv[1][1])[0] if prof else None
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs")
    peak_src = "measured (MEASURED_PEAKS.json hbm_gbs)" if peak else "fallback 6800 GB/s"
    peak = peak or 6800.0
    algo_bytes_step = sum(v[2] for v in prof.values()) / prof_steps if prof else None
    roof = None
    if dom and prec == 8:
        # FP64 FFTs on GB300 are bound by the FP64 pipe, not HBM: compare the
        # FFT flop rate (2.5 N log2 N per r2c direction, the usual count)
        # with a FP64 peak measured here (float64 GEMM through torch).
        import math
        fp64_peak = measure_fp64_tflops(dev)
        flops = 2 * 2.5 * npts * math.log2(npts)
        achieved = flops / (ms_max * 1e-3) / 1e12
        d = passes[dom]
        roof = {"bound": "fp64", "kernel": "all six axis passes of the step", "achieved": round(achieved, 3),
                "peak": round(fp64_peak, 3), "unit": "TFLOP/s", "frac": round(achieved / fp64_peak, 4),
                "traffic": read_traffic(args.workload, dom),
                "peak_source": "measured in this run: float64 GEMM 4096^3 (torch), best of 3",
                "hbm": {"dominant_pass": dom, "achieved_gbs": round(d["gbs"], 1), "peak_gbs": peak,
                        "frac": round(d["gbs"] / peak, 4)}}
    elif dom:
        d = passes[dom]
        traffic = read_traffic(args.workload + ("" if args.form == "plain" else ":" + args.form), dom)
        roof = {"bound": "hbm", "kernel": "axis pass %s" % dom, "achieved": round(d["gbs"], 1),
                "peak": peak, "unit": "GB/s", "frac": round(d["gbs"] / peak, 4),
                "traffic": traffic,
                "traffic_source": ("committed profile (profiles/dram_traffic.txt: ncu dram bytes of reduced grids "
                                   "of the same kernel, scaled to a full launch), not measured in this run")
                if traffic is not None else "no ncu figure committed for this workload and pass",
                "peak_source": peak_src,
                "step_frac": round(algo_bytes_step / (ms_max * 1e-3) / 1e9 / peak, 4)}

    # end to end through the C ABI with host buffers
    hb = HostBuffers(local)
    xh = hb.empty(x.shape, x.dtype)
    xh.copy_(x)
    yh = hb.empty(x.shape, x.dtype)
    xd = torch.empty_like(x)
    e2e_steps = max(3, min(args.steps, 20))
    # On these machines the host link can run at a fraction of its rate in
    # one direction, or in both at once, for a minute or more after other
    # work on the machine (the other direction at full speed).  Wait, at most
    # 90 s, until no reading of a short link test (each direction alone, both
    # at once) is below 60 % of the faster direction; the wait and the link
    # state are reported with the figure.
    def link_degraded(lk):
        return min(lk["h2d"], lk["d2h"], lk["both_each"]) < 0.6 * max(lk["h2d"], lk["d2h"])

    link = link_gbs(xh, xd, stream, host2=yh)
    t_settle = time.time()
    while link_degraded(link) and time.time() - t_settle < 90.0:
        time.sleep(2.0)
        link = link_gbs(xh, xd, stream, reps=2, host2=yh)
    settle_s = round(time.time() - t_settle, 1)

    def e2e_step():
        xd.copy_(xh, non_blocking=True)
        eng.r2c(xd, spec, stream)
        eng.c2r(spec, y, stream)
        yh.copy_(y, non_blocking=True)

    e2e_step()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(e2e_steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    serial_ms = max_over_ranks(e0.elapsed_time(e1) / e2e_steps)

    # The same steps as an application would stream them: step i's input
    # copy (own stream) and step i-1's result copy (own stream) overlap step
    # i's transforms; inputs and results are double-buffered, the transforms
    # of consecutive steps stay in order on one stream (they share the
    # engine's work area).  Every step still copies its whole input in from
    # pinned host memory and its whole result out.
    s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    xd2 = [xd, torch.empty_like(x)]
    y2 = [y, torch.empty_like(y)]
    yh2 = [yh, hb.empty(yh.shape, yh.dtype)]

    copy_ms = {"h2d": [], "d2h": []}

    def pipelined(nsteps, t0=None, t1=None):
        ev_in = [torch.cuda.Event() for _ in range(nsteps)]
        ev_comp = [torch.cuda.Event() for _ in range(nsteps)]
        ev_out = [torch.cuda.Event() for _ in range(nsteps)]
        # every copy's own duration: the link bandwidth this window really got
        c_in = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
        c_out = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
        if t0 is not None:
            t0.record(s_in)
        for i in range(nsteps):
            b = i % 2
            if i >= 2:
                s_in.wait_event(ev_comp[i - 2])  # xd2[b] read by step i-2
            c_in[i][0].record(s_in)
            with torch.cuda.stream(s_in):
                xd2[b].copy_(xh, non_blocking=True)
            c_in[i][1].record(s_in)
            ev_in[i].record(s_in)
            stream.wait_event(ev_in[i])
            if i >= 2:
                stream.wait_event(ev_out[i - 2])  # y2[b] copied out by step i-2
            eng.r2c(xd2[b], spec, stream)
            eng.c2r(spec, y2[b], stream)
            ev_comp[i].record(stream)
            s_out.wait_event(ev_comp[i])
            c_out[i][0].record(s_out)
            with torch.cuda.stream(s_out):
                yh2[b].copy_(y2[b], non_blocking=True)
            c_out[i][1].record(s_out)
            ev_out[i].record(s_out)
        if t1 is not None:
            s_out.wait_event(ev_comp[nsteps - 1])
            t1.record(s_out)
        torch.cuda.synchronize()
        copy_ms["h2d"].append(sum(a.elapsed_time(b) for a, b in c_in) / nsteps)
        copy_ms["d2h"].append(sum(a.elapsed_time(b) for a, b in c_out) / nsteps)
        return (nsteps - 1) % 2

    pipelined(2)
    torch.cuda.synchronize()
    # five repetitions of at least 10 steps each, the median reported: the
    # host link is shared with the machine's other GPUs, so one repetition
    # can be slowed by traffic that is not this job's
    pipe_steps = max(10, e2e_steps)
    reps = []
    for _ in range(5):
        barrier()
        torch.cuda.synchronize()
        last = pipelined(pipe_steps, e0, e1)
        torch.cuda.synchronize()
        barrier()
        reps.append(max_over_ranks(e0.elapsed_time(e1) / pipe_steps))
    e2e_ms = sorted(reps)[len(reps) // 2]
    med = reps.index(e2e_ms)
    observed = {k: round(x.numel() * x.element_size() / (v[1 + med] * 1e-3) / 1e9, 1) for k, v in copy_ms.items()}
    same = bool(torch.equal(yh2[last], yh2[1 - last]))  # deterministic: every step's result alike
    link_after = link_gbs(xh, xd, stream, host2=yh)
    placement = hb.placement()
    del xh, yh, yh2
    hb.release()
    e2e = {"value": round(total_pts / (e2e_ms * 1e-3) / 1e9, 3), "unit": "GPts/s",
           "ms_per_step": round(e2e_ms, 3),
           "h2d_bytes_per_step": x.numel() * x.element_size(),
           "d2h_bytes_per_step": y.numel() * y.element_size(),
           "form": "copies of step i+1 / i-1 overlap the transforms of step i (double-buffered); median of "
                   "5 repetitions of %d steps" % pipe_steps,
           "repetitions_ms": [round(v, 3) for v in reps],
           "results_identical_across_steps": same,
           "host_link_gbs": link,
           "host_link_gbs_after": link_after,
           "host_buffers": placement,
           "link_settle_s": settle_s,
           "copy_gbs_during_e2e": observed,
           "host_cpus": "%d CPUs on the GPU's NUMA node (%s)" % (len(cpus), "bound" if gpu_local_cpus(local) else
                                                                 "node unknown: not bound"),
           "link_bound_ms": round(max(x.numel() * x.element_size() / (link["both_each"] * 1e9),
                                      y.numel() * y.element_size() / (link["both_each"] * 1e9)) * 1e3, 3),
           "serial": {"value": round(total_pts / (serial_ms * 1e-3) / 1e9, 3), "ms_per_step": round(serial_ms, 3),
                      "form": "copy in, r2c, c2r, copy out on one stream"}}

    out = None
    if rank == 0:
        acc = {}
        if not args.no_accuracy:
            step()
            torch.cuda.synchronize()
            rel, mx = fp64_accuracy(x, spec, fmt)
            yy = (y.double() / npts - x.double())
            rt = float(torch.linalg.vector_norm(yy) / torch.linalg.vector_norm(x.double()))
            acc = {"rel_l2_vs_fp64": rel, "max_abs_rel_vs_fp64": mx, "round_trip_rel_l2": rt,
                   "fp64_reference": "pocketfft (scipy.fft) FP64 on the same input"}
        cpu = None
        if not args.no_cpu:
            cpu = cpu_baseline(nx, ny, nz, fmt, prec, steps=args.cpu_steps, warmup=1,
                               x=x.cpu().numpy())
        out = {
            "metric": METRIC,
            "value": round(value, 3),
            "unit": "GPts/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(ms_max, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32" if prec == 4 else "f64",
            "data": "synthetic: %s" % ("seeded N(0,1) + 8 sinusoid modes of amplitude 10" if kind == "gauss_modes"
                                       else "seeded uniform [-1,1)"),
            "config": {"workload": "r2c+c2r round trip %dx%dx%d %s %s" % (
                nx, ny, nz, "fp32" if prec == 4 else "fp64", "PHYSICAL_IN_X" if fmt == 1 else "PHYSICAL_IN_Z"),
                "name": args.workload, "nx": nx, "ny": ny, "nz": nz, "form": args.form,
                "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas (one grid per GPU)"},
            "roofline": roof,
            "passes": {k: {kk: (round(vv, 4) if isinstance(vv, float) else vv) for kk, vv in v.items()}
                       for k, v in passes.items()},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk,
            "accuracy": acc,
        }
        print(json.dumps(out), flush=True)
    eng.close()
    d = _dist()
    if d is not None:
        d.destroy_process_group()
    return out


def batch_dims(count=64, seed=6):
    """64 grids, each dimension drawn from {32,48,64,96,128,192,256} (seed 6),
    PHYSICAL_IN_X or PHYSICAL_IN_Z by a seeded coin."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        nx, ny, nz = (int(v) for v in rng.choice([32, 48, 64, 96, 128, 192, 256], size=3))
        fmt = 1 if rng.random() < 0.5 else 3
        out.append((nx, ny, nz, fmt))
    return out


def run_batched(args):
    """Batched uneven grids: forward + backward of 64 FP32 grids per step,
    timed as one persistent launch replayed from a CUDA graph (value) and as
    the per-grid launch loop (reported beside it)."""
    import numpy as np
    import torch
    import gbfft
    world, rank, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    gbfft.lib()
    dims = batch_dims()
    rng = np.random.default_rng(7)
    items = []
    batch = gbfft.Batch()
    npts = 0
    for nx, ny, nz, fmt in dims:
        e = gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE)
        x = torch.from_numpy(rng.uniform(-1, 1, (nz, ny, nx)).astype(np.float32)).to(dev)
        s = e.empty_spectral(device=dev)
        batch.add(e, x, s)
        items.append((e, x, s, fmt))
        npts += nx * ny * nz
    stream = torch.cuda.Stream(dev)
    info = batch.info()
    # per-grid error of the forward spectrum against FP64 (before timing)
    x0 = [x.clone() for _, x, _, _ in items]
    batch.run(1, stream)
    stream.synchronize()
    errs = []
    for (e, x, s, fmt) in items:
        xd = x.double().cpu().numpy()
        ref = np.fft.rfftn(xd, axes=(0, 1, 2)) if fmt == 1 else np.fft.rfftn(xd, axes=(2, 1, 0))
        errs.append(float(np.linalg.norm(s.cpu().numpy() - ref) / np.linalg.norm(ref)))

    def timed(fn, steps, warm):
        for _ in range(warm):
            fn()
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = gbfft.launch_count()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1) / steps, gbfft.launch_count() - l0

    batch.graph_build(stream)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    t0 = time.time()
    ms_graph, _ = timed(lambda: batch.graph_launch(stream), args.steps, args.warmup)
    t1 = time.time()
    # kernels per step: one persistent launch, or every pass of every grid
    l0 = gbfft.launch_count()
    batch.run(3, stream)
    stream.synchronize()
    per_step = gbfft.launch_count() - l0
    launches = per_step * args.steps
    batch.status()
    batch.set_persistent(False)
    batch.graph_build(stream)
    ms_loop_graph, _ = timed(lambda: batch.graph_launch(stream), args.steps, args.warmup)
    ms_loop, loop_launches = timed(lambda: (batch.forward(stream), batch.backward(stream)), args.steps,
                                   args.warmup)
    for (e, x, s, fmt), xr in zip(items, x0):
        x.copy_(xr)
    clocks.stop()
    for (e, x, s, fmt), xr in zip(items, x0):
        x.copy_(xr)
    value = npts / (ms_graph * 1e-3) / 1e9
    out = {"metric": METRIC, "value": round(value, 3), "unit": "GPts/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_graph, 4),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic: seeded uniform [-1,1)",
           "config": {"workload": "batched uneven grids: 64 FP32 grids, dims from {32..256}, mixed X/Z, "
                                  "r2c+c2r per step", "name": BATCH_WORKLOAD, "points": npts,
                      "persistent": info["persistent"],
                      "l2": "no flush (total working set %.0f MB)" % (npts * 4 * 3 / 1e6)},
           "batch": {"persistent_graph_ms": round(ms_graph, 4), "per_grid_loop_graph_ms": round(ms_loop_graph, 4),
                     "per_grid_loop_ms": round(ms_loop, 4), "launches_per_step_persistent": per_step,
                     "launches_per_step_loop": loop_launches / args.steps,
                     "speedup_vs_loop": round(ms_loop / ms_graph, 3),
                     "per_grid_rel_l2_vs_fp64_max": max(errs), "per_grid_rel_l2_vs_fp64_median": sorted(errs)[len(errs) // 2]},
           "gpu_launches": int(launches), "clocks": clocks.summary(t0, t1)}
    if rank == 0:
        print(json.dumps(out), flush=True)
    batch.close()
    return out


def measure_fp64_tflops(dev, n=4096):
    """FP64 throughput of this GPU, from a float64 GEMM (2 n^3 flops)."""
    import torch
    a = torch.randn((n, n), dtype=torch.float64, device=dev)
    b = torch.randn((n, n), dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = None
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) * 1e-3
        best = t if best is None or t < best else best
    return 2.0 * n ** 3 / best / 1e12


def read_traffic(workload, kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (profiles/dram_traffic.txt: `workload kernel bytes_per_launch`)."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 3 and not line.startswith("#") and parts[0] == workload and parts[1] == kernel:
                return float(parts[2])
    except Exception:
        pass
    return None


def run_dtt(args):
    """Real-to-real transforms: one step = decomp_2d_dtt_3d_r2r forward then
    backward (6 axis passes, each one read and one write of the real array)."""
    import torch
    import numpy as np
    import gbfft
    from oracle import dtt as D
    world, rank, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    nx, ny, nz, prec, kinds = DTT_WORKLOADS[args.workload]
    rdt = torch.float32 if prec == 4 else torch.float64
    gbfft.lib()
    eng = gbfft.Dtt(1, nx, ny, nz, list(kinds), prec=prec)
    rng = np.random.default_rng(7)
    a = rng.uniform(-1, 1, (nz, ny, nx))
    x = torch.from_numpy(a).to(rdt).to(dev)
    y = torch.empty_like(x)
    stream = torch.cuda.current_stream(dev)
    npts = nx * ny * nz

    def step():
        eng.r2r(x, y, -1, stream)
        eng.r2r(y, x, 1, stream)

    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    l0 = gbfft.launch_count()
    t_wall0 = time.time()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    t_wall1 = time.time()
    barrier()
    launches = gbfft.launch_count() - l0
    clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    value = sum_over_ranks(npts) / (ms * 1e-3) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs") or 6800.0
    bytes_step = 6 * 2 * npts * (4 if prec == 4 else 8)
    achieved = bytes_step / (ms * 1e-3) / 1e9
    # end to end: input from pinned host memory, result back, every step
    xh = torch.empty(x.shape, dtype=rdt, pin_memory=True)
    xh.copy_(torch.from_numpy(a).to(rdt))
    yh = torch.empty_like(xh, pin_memory=True)
    e2e_steps = max(3, min(args.steps, 20))

    def e2e_step():
        x.copy_(xh, non_blocking=True)
        eng.r2r(x, y, -1, stream)
        eng.r2r(y, x, 1, stream)
        yh.copy_(x, non_blocking=True)

    e2e_step()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(e2e_steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1) / e2e_steps)
    out = None
    if rank == 0:
        # accuracy: forward transform against the FP64 oracle, round trip
        x.copy_(torch.from_numpy(a).to(rdt))
        eng.r2r(x, y, -1, stream)
        torch.cuda.synchronize()
        cfg = D.config(kinds)
        acc = {}
        if not args.no_accuracy:
            sub = (slice(0, 16), slice(None), slice(None))  # 16 z-planes of the oracle's dense matrices
            _, ref = D.dtt_3d_r2r(a, 1, cfg, -1)
            got = y.double().cpu().numpy()
            acc["rel_l2_vs_fp64"] = float(np.linalg.norm((got - ref)[sub]) / np.linalg.norm(ref[sub]))
        cpu = None
        if not args.no_cpu:
            t0 = time.time()
            reps = 0
            while time.time() - t0 < min(args.cpu_seconds, 10.0) or reps == 0:
                D.dtt_3d_r2r(a, 1, cfg, -1)
                reps += 1
            dt = (time.time() - t0) / reps
            cpu = {"value": round(npts / (2 * dt) / 1e9, 5), "unit": "GPts/s", "cores": os.cpu_count() or 1,
                   "kind": "port",
                   "sample": "oracle forward transform (dense float64 matrices, numpy with its BLAS threads) on "
                             "the full grid, %d repetitions; a round trip counted as twice its time" % reps}
        out = {
            "metric": "3D r2r (DCT/DST) forward+backward GPts/s & %HBM roofline",
            "value": round(value, 3), "unit": "GPts/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if prec == 4 else "f64",
            "data": "synthetic: seeded uniform [-1,1)",
            "config": {"workload": "r2r DCT-II on x, y, z (default windows) forward+backward %dx%dx%d %s" % (
                nx, ny, nz, "fp32" if prec == 4 else "fp64"), "name": args.workload, "nx": nx, "ny": ny,
                "nz": nz, "kinds": list(kinds), "l2": "inputs larger than L2" if npts * (prec) > 130e6
                else "inputs smaller than L2 (no flush)", "parallelism": "replicas (one grid per GPU)"},
            "roofline": {"bound": "hbm", "kernel": "all six r2r axis passes of the step",
                         "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": None,
                         "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)"},
            "cpu_baseline": cpu,
            "e2e": {"value": round(npts / (e2e_ms * 1e-3) / 1e9, 3), "unit": "GPts/s",
                    "ms_per_step": round(e2e_ms, 3),
                    "h2d_bytes_per_step": x.numel() * x.element_size(),
                    "d2h_bytes_per_step": x.numel() * x.element_size()},
            "gpu_launches": int(launches),
            "clocks": clocks.summary(t_wall0, t_wall1),
            "accuracy": acc,
        }
        print(json.dumps(out), flush=True)
    eng.close()
    return out


def run_c2c_chain(args):
    """Transposes plus c2c on 256^3: one step = a complex64 c2c forward +
    backward through the C ABI (value, GPts/s); beside it the four one-rank
    transposes (x->y->z->y->x) on real64 and complex128 arrays, timed as
    copies (GB/s against the copy peak) and checked bit for bit."""
    import torch
    import numpy as np
    import gbfft
    from oracle import oracle as O
    world, rank, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n = 256
    npts = n ** 3
    gbfft.lib()
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(9)
    a = (rng.uniform(-1, 1, (n, n, n)) + 1j * rng.uniform(-1, 1, (n, n, n))).astype(np.complex64)
    x = torch.from_numpy(a).to(dev)
    y = torch.empty_like(x)
    eng = gbfft.Engine(gbfft.PHYSICAL_IN_X, n, n, n, prec=gbfft.PREC_SINGLE)

    def step():
        eng.c2c(x, y, gbfft.FORWARD, stream)
        eng.c2c(y, x, gbfft.BACKWARD, stream)

    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    x.copy_(torch.from_numpy(a))
    barrier()
    torch.cuda.synchronize()
    l0 = gbfft.launch_count()
    t_wall0 = time.time()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    t_wall1 = time.time()
    barrier()
    launches = gbfft.launch_count() - l0
    # per-pass device times, in steps of their own (events recorded by the library)
    prof_steps = max(1, min(args.steps, 10))
    eng.set_profiling(True)
    for _ in range(prof_steps):
        step()
    torch.cuda.synchronize()
    prof = eng.profile()
    eng.set_profiling(False)
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    value = sum_over_ranks(npts) / (ms * 1e-3) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs") or 6800.0
    bytes_step = 6 * 2 * npts * 8  # six passes, each one read and one write of the complex64 array
    # the transpose chain, real64 and complex128 (4 identity copies each)
    chains = {}
    reps = max(3, min(args.steps, 20))
    for name, dt, cplx in (("real64", torch.float64, 0), ("complex128", torch.complex128, 1)):
        src = torch.from_numpy(rng.uniform(-1, 1, (n, n, n))).to(dt).to(dev) if not cplx else \
            torch.from_numpy(rng.uniform(-1, 1, (n, n, n)) + 1j * rng.uniform(-1, 1, (n, n, n))).to(dt).to(dev)
        bufs = [torch.empty_like(src) for _ in range(4)]

        def chain():
            seq = [src] + bufs
            for k, kind in enumerate((gbfft.X_TO_Y, gbfft.Y_TO_Z, gbfft.Z_TO_Y, gbfft.Y_TO_X)):
                gbfft.transpose(kind, seq[k], seq[k + 1], n, n, n, cplx, gbfft.PREC_DOUBLE, stream)

        for _ in range(3):
            chain()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            chain()
        e1.record(stream)
        torch.cuda.synchronize()
        cms = max_over_ranks(e0.elapsed_time(e1) / reps)
        cbytes = 4 * 2 * src.numel() * src.element_size()
        chains[name] = {"ms_per_chain": round(cms, 4), "gbs": round(cbytes / (cms * 1e-3) / 1e9, 1),
                        "frac": round(cbytes / (cms * 1e-3) / 1e9 / peak, 4), "bytes_per_chain": cbytes,
                        "bit_exact": bool(torch.equal(bufs[-1], src))}
    # end to end: input from pinned host memory, result back, every step
    xh = torch.empty(x.shape, dtype=x.dtype, pin_memory=True)
    xh.copy_(torch.from_numpy(a))
    yh = torch.empty_like(xh, pin_memory=True)

    def e2e_step():
        x.copy_(xh, non_blocking=True)
        eng.c2c(x, y, gbfft.FORWARD, stream)
        eng.c2c(y, x, gbfft.BACKWARD, stream)
        yh.copy_(x, non_blocking=True)

    e2e_step()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1) / reps)
    clocks.stop()
    out = None
    if rank == 0:
        acc = {}
        if not args.no_accuracy:
            x.copy_(torch.from_numpy(a))
            eng.c2c(x, y, gbfft.FORWARD, stream)
            torch.cuda.synchronize()
            ref = np.fft.fftn(a.astype(np.complex128))
            acc["rel_l2_vs_fp64"] = float(np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref))
            acc["fp64_reference"] = "numpy pocketfft FP64 on the same input"
        cpu = None
        if not args.no_cpu:
            threads = O.set_threads(os.cpu_count() or 1)
            O.fft3d_c2c(a, O.PHYSICAL_IN_X, O.FORWARD, prec="s")  # warm-up
            t0 = time.time()
            r = 0
            while r < 2:
                f = O.fft3d_c2c(a, O.PHYSICAL_IN_X, O.FORWARD, prec="s")
                O.fft3d_c2c(f, O.PHYSICAL_IN_X, O.BACKWARD, prec="s")
                r += 1
            dt = (time.time() - t0) / r
            cpu = {"value": round(npts / dt / 1e9, 5), "unit": "GPts/s", "cores": threads, "kind": "port",
                   "ms_per_round_trip": round(dt * 1e3, 1),
                   "sample": "oracle (restated generic backend, single build), OpenMP over lines: whole c2c "
                             "forward + backward round trips of the full grid, 1 warm-up then the mean of 2"}
        passes = {}
        for k, (nl, tms, by) in prof.items():
            per = tms / nl
            passes[k] = {"launches_per_step": nl / prof_steps, "ms_per_launch": round(per, 4),
                         "gbs": round(by / (tms * 1e-3) / 1e9, 1), "bytes_per_launch": by / nl}
        dom = max(passes, key=lambda k: passes[k]["ms_per_launch"] * passes[k]["launches_per_step"]) \
            if passes else None
        out = {
            "metric": "3D c2c forward+backward GPts/s (complex64) & %HBM roofline; transpose chain bit-exact",
            "value": round(value, 3), "unit": "GPts/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded uniform [-1,1) real and imaginary parts",
            "config": {"workload": "transposes x->y->z->y->x (real64, complex128) then c2c forward+backward "
                                   "256x256x256 complex64", "name": args.workload, "nx": n, "ny": n, "nz": n,
                       "l2": "arrays of 134-268 MB, around the 129 MB L2 (no flush)",
                       "parallelism": "replicas (one grid per GPU)"},
            "roofline": {"bound": "hbm", "kernel": ("axis pass %s" % dom) if dom else "six c2c axis passes",
                         "achieved": passes[dom]["gbs"] if dom else None, "peak": peak, "unit": "GB/s",
                         "frac": round(passes[dom]["gbs"] / peak, 4) if dom else None, "traffic": None,
                         "step_frac": round(bytes_step / (ms * 1e-3) / 1e9 / peak, 4),
                         "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)"},
            "passes": passes,
            "transposes": chains,
            "cpu_baseline": cpu,
            "e2e": {"value": round(npts / (e2e_ms * 1e-3) / 1e9, 3), "unit": "GPts/s",
                    "ms_per_step": round(e2e_ms, 3),
                    "h2d_bytes_per_step": x.numel() * x.element_size(),
                    "d2h_bytes_per_step": x.numel() * x.element_size()},
            "gpu_launches": int(launches),
            "clocks": clocks.summary(t_wall0, t_wall1),
            "accuracy": acc,
        }
        print(json.dumps(out), flush=True)
    eng.close()
    return out


def run_reference(args):
    """The reference arm: the reference's CPU path for this workload -- the
    oracle, a restatement of its generic backend (the Fortran reference
    cannot be built on these machines) -- on all host cores.  Every step is
    one whole r2c + c2r round trip of the full grid; W untimed steps, then
    the mean of K timed ones."""
    world, rank, local = dist_env()
    if rank != 0:
        return None
    if args.workload not in WORKLOADS:
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the complex-FFT workloads; "
                          "%s has no CPU reference run" % args.workload}), flush=True)
        return None
    nx, ny, nz, fmt, prec, kind = WORKLOADS[args.workload]
    x = host_input(nx, ny, nz, prec)
    t0 = time.time()
    sec, threads = cpu_round_trips(x, fmt, prec, args.steps, args.warmup)
    wall = time.time() - t0
    v = nx * ny * nz / sec / 1e9
    desc = ("oracle (restated generic backend, Glassman FFT, %s build), OpenMP over lines on %d host threads: "
            "each step one whole r2c+c2r round trip of the full grid (every line of all 6 passes)"
            % ("double" if prec == 8 else "single", threads))
    out = {"metric": METRIC, "value": round(v, 5), "unit": "GPts/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sec * 1e3, 2),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32" if prec == 4 else "f64", "data": "synthetic: seeded N(0,1) host field (the line FFT "
           "cost does not depend on the values)", "impl": "reference",
           "config": {"workload": "r2c+c2r round trip %dx%dx%d %s %s" % (
               nx, ny, nz, "fp32" if prec == 4 else "fp64", "PHYSICAL_IN_X" if fmt == 1 else "PHYSICAL_IN_Z"),
               "name": args.workload, "nx": nx, "ny": ny, "nz": nz,
               "parallelism": "OpenMP threads over lines on the host cores"},
           "cpu_baseline": {"value": round(v, 5), "unit": "GPts/s", "cores": threads, "kind": "port",
                            "sample": desc},
           "timed_wall_s": round(wall, 2),
           "e2e": {"value": round(v, 5), "unit": "GPts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 200; the reference arm's steps are whole CPU round trips of "
                         "about 2 s each: default 20)")
    ap.add_argument("--warmup", type=int, default=None, help="untimed steps first (default 10; reference arm 3)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD,
                    choices=sorted(WORKLOADS) + [BATCH_WORKLOAD, C2C_WORKLOAD] + sorted(DTT_WORKLOADS))
    ap.add_argument("--form", default="plain", choices=["plain", "split", "split_tc"],
                    help="plain FP32/FP64 stages, split-FP16 tensor-core radix-16 stages on mma.sync (split), "
                         "or with the strided 1024-point passes on tcgen05 (split_tc); FP32 only")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="CPU time budget of the r2r workloads' oracle leg")
    ap.add_argument("--cpu-steps", type=int, default=2,
                    help="timed whole round trips of the CPU leg (after one warm-up)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 20 if args.impl == "reference" else 200
    if args.warmup is None:
        args.warmup = 3 if args.impl == "reference" else 10
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == BATCH_WORKLOAD:
        run_batched(args)
    elif args.workload in DTT_WORKLOADS:
        run_dtt(args)
    elif args.workload == C2C_WORKLOAD:
        run_c2c_chain(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
