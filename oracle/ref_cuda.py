"""Launch cctpy's own CUDA tracking kernel on the current GPU (test and benchmark
infrastructure, not part of the product).

``ref_cuda_build.py`` compiles the kernel source that cctpy's ``GPU_ACCELERATOR`` assembles
into device-only cubins under ``oracle/_ref/``; this module loads them with the CUDA driver
API (through ctypes on libcuda, so nothing is compiled where it runs) and launches
``track_multi_particle_beamline_for_magnet_with_multi_qs`` exactly as cctpy's host code does
(gpu_accelerator.py:1931-2031): one block of ``block_dim_x`` threads per beamline, the
per-beamline segment arrays padded to ``max_current_element_number`` x 3 and the QS records
to ``max_qs_datas_length`` x 16, every beamline given the same particles, the particle
records written back in place.  The tests use it to pin the FP64 engine against cctpy's own
GPU kernel on the same device, and the benchmark to time cctpy's GPU path beside ours.
"""
from __future__ import annotations

import ctypes
import json
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
META = os.path.join(REF_DIR, "cctpy_cuda.json")
# cctpy's two multi-beamline kernels (gpu_accelerator.py:1023-1063) and their arguments
KERNELS = {
    "multi_qs": ("track_multi_particle_beamline_for_magnet_with_multi_qs",
                 ("distance", "footstep", "kls", "p0s", "n_ce", "qs", "n_qs", "particles", "n_p")),
    "single_qs": ("track_multi_particle_beamline_for_magnet_with_single_qs",
                  ("distance", "footstep", "kls", "p0s", "n_ce", "qs", "particles", "n_p")),
}


def available() -> bool:
    return os.path.isfile(META)


class _Driver:
    """The handful of CUDA driver calls the launch needs, on the context torch made current."""

    def __init__(self):
        self.lib = ctypes.CDLL("libcuda.so.1")
        L = self.lib
        L.cuInit.argtypes = [ctypes.c_uint]
        L.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        L.cuModuleUnload.argtypes = [ctypes.c_void_p]
        L.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        L.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [
            ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p)]
        L.cuGetErrorName.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        self.check(L.cuInit(0), "cuInit")

    def check(self, rc: int, what: str) -> None:
        if rc != 0:
            name = ctypes.c_char_p()
            self.lib.cuGetErrorName(rc, ctypes.byref(name))
            raise RuntimeError(f"{what} failed: {name.value.decode() if name.value else rc}")


def pack(designs, particles: np.ndarray, max_ce: int, max_qs: int, dtype, single_qs: bool = False) -> dict:
    """Host arrays in cctpy's GPU layout (gpu_accelerator.py:1953-2016).  ``designs``: per
    beamline (kls (n, 3), p0s (n, 3), qs (k, 16)); ``particles``: (n_p, 10) records, given to
    every beamline; ``max_ce`` / ``max_qs``: the kernel's compiled capacities.  single_qs:
    the layout of cctpy's single-QS kernel (gpu_accelerator.py:1834-1874): one 16-number
    record per beamline, the beamline's last QS (cctpy's host loop keeps overwriting it), and
    a beamline without a QS refused (cctpy's concatenation of its None fails there)."""
    D = len(designs)
    parts = np.ascontiguousarray(particles, dtype=np.float64).reshape(-1, 10)
    n_p = parts.shape[0]
    if D < 1 or n_p < 1:
        raise ValueError("need at least one beamline and one particle")
    kls = np.zeros((D, 3 * max_ce), dtype)
    p0s = np.zeros((D, 3 * max_ce), dtype)
    qs = np.zeros((D, 16 * max_qs), dtype)
    n_ce = np.zeros(D, np.int32)
    n_qs = np.zeros(D, np.int32)
    for d, (k, p, q) in enumerate(designs):
        k = np.asarray(k, np.float64).reshape(-1)
        p = np.asarray(p, np.float64).reshape(-1)
        q = np.asarray(q, np.float64).reshape(-1)
        if k.size % 3 or k.size != p.size or q.size % 16:
            raise ValueError(f"beamline {d}: kls and p0s must be (n, 3) alike and QS records 16 doubles")
        if k.size > 3 * max_ce or q.size > 16 * max_qs:
            raise ValueError(f"beamline {d} exceeds cctpy's GPU capacities ({max_ce} current elements, "
                             f"{max_qs} QS)")
        kls[d, :k.size] = k
        p0s[d, :p.size] = p
        qs[d, :q.size] = q
        n_ce[d] = k.size // 3
        n_qs[d] = q.size // 16
    if single_qs:
        if not n_qs.all():
            raise ValueError("cctpy's single-QS kernel needs a QS in every beamline")
        qs = np.stack([qs[d, 16 * (n_qs[d] - 1):16 * n_qs[d]] for d in range(D)])
    return dict(kls=kls, p0s=p0s, n_ce=n_ce, qs=qs, n_qs=n_qs,
                particles=np.tile(parts, (D, 1)).astype(dtype), n_p=np.array([n_p], np.int32))


class ReferenceCudaTracker:
    """cctpy's GPU tracking kernel in one of the built configurations ("f32": FLOAT32 x 1024
    threads, "f64": FLOAT64 x 512 threads, both with cctpy's default capacities; "f32_700k",
    "f64_700k": the same with room for 700 000 current elements a beamline), loaded on the
    current CUDA device.  kernel: "multi_qs" (every QS of a beamline, the kernel cctpy's
    track_multi_particle_beamline_for_magnet_with_multi_qs launches) or "single_qs"."""

    def __init__(self, precision: str = "f32", kernel: str = "multi_qs"):
        import torch
        if not available():
            raise FileNotFoundError("cctpy's CUDA kernels are not built (oracle/ref_cuda_build.py)")
        with open(META) as f:
            meta = json.load(f)
        cfg = meta["configs"][precision]
        self.precision = precision
        self.block = int(cfg["block"])
        self.max_ce = int(cfg["max_current_element_number"])
        self.max_qs = int(cfg["max_qs_datas_length"])
        single = int(cfg["float_bytes"]) == 4
        self.np_dtype = np.float32 if single else np.float64
        self.torch_dtype = torch.float32 if single else torch.float64
        torch.zeros(1, device="cuda")                    # torch's primary context is current
        self.drv = _Driver()
        self.module = ctypes.c_void_p()
        self.drv.check(self.drv.lib.cuModuleLoad(ctypes.byref(self.module),
                                                 os.path.join(REF_DIR, cfg["cubin"]).encode()), "cuModuleLoad")
        self.single_qs = kernel == "single_qs"
        name, self.args = KERNELS[kernel]
        self.fn = ctypes.c_void_p()
        self.drv.check(self.drv.lib.cuModuleGetFunction(ctypes.byref(self.fn), self.module, name.encode()),
                       "cuModuleGetFunction")

    def close(self) -> None:
        if self.module:
            self.drv.lib.cuModuleUnload(self.module)
            self.module = ctypes.c_void_p()

    def pack(self, designs, particles: np.ndarray) -> dict:
        return pack(designs, particles, self.max_ce, self.max_qs, self.np_dtype, self.single_qs)

    def upload(self, host: dict, distance: float, footstep: float) -> dict:
        import torch
        dev = {k: torch.from_numpy(v).to("cuda") for k, v in host.items()}
        dev["distance"] = torch.tensor([distance], dtype=self.torch_dtype, device="cuda")
        dev["footstep"] = torch.tensor([footstep], dtype=self.torch_dtype, device="cuda")
        return dev

    def launch(self, dev: dict) -> None:
        """One launch on torch's current stream: grid = beamlines, block = block_dim_x."""
        import torch
        ptrs = [ctypes.c_void_p(dev[k].data_ptr()) for k in self.args]
        params = (ctypes.c_void_p * len(ptrs))(*[ctypes.cast(ctypes.pointer(p), ctypes.c_void_p) for p in ptrs])
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        D = int(dev["n_ce"].shape[0])
        self.drv.check(self.drv.lib.cuLaunchKernel(self.fn, D, 1, 1, self.block, 1, 1, 0, stream, params, None),
                       "cuLaunchKernel")

    def track(self, designs, particles: np.ndarray, distance: float, footstep: float):
        """Track every particle through every beamline.  Returns (records (D, n_p, 10) float64,
        kernel seconds (CUDA events), call seconds: packing, copies in, kernel, copy out)."""
        import torch
        t0 = time.perf_counter()
        host = self.pack(designs, particles)
        dev = self.upload(host, distance, footstep)
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        self.launch(dev)
        stop.record()
        out = dev["particles"].to("cpu").numpy().astype(np.float64)
        torch.cuda.synchronize()
        t_call = time.perf_counter() - t0
        D, n_p = host["n_ce"].shape[0], int(host["n_p"][0])
        return out.reshape(D, n_p, 10), start.elapsed_time(stop) / 1e3, t_call
