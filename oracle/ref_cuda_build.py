"""Recipe: compile cctpy's own CUDA tracking kernels for sm_103a, for a same-GPU comparison.

Test and benchmark infrastructure, not part of the product.  cctpy's GPU path is a CUDA
source string that ``GPU_ACCELERATOR.__init__`` assembles
(final_code/packages/gpu_accelerator.py:100-1078) and pycuda compiles at every call
(``SourceModule``, gpu_accelerator.py:1933).  This recipe imports that module unmodified
from a cctpy checkout, takes the string for the two configurations cctpy's GPU speed test and
documentation use (FLOAT32 with 1024 threads a block, FLOAT64 with 512;
gpu_accelerator.py:54-70), wraps it in ``extern "C"`` as pycuda does, and compiles it with
nvcc into device-only cubins:

    oracle/_ref/cctpy_track_f32.cubin, oracle/_ref/cctpy_track_f64.cubin,
    oracle/_ref/cctpy_track_f32_700k.cubin, oracle/_ref/cctpy_track_f64_700k.cubin,
    oracle/_ref/cctpy_cuda.json (block sizes, array capacities, registers, source hash)

The last two have room for 700 000 current elements a beamline (the
``max_current_element_number`` constructor argument): the gantry-section and population
designs (up to ~625 000 segments) exceed cctpy's default of 240 000.

The source is written to a temporary directory outside the repository and deleted after the
compile; only the device binaries and their description are kept (``oracle/_ref/`` is
git-ignored).  ``oracle/ref_cuda.py`` loads and launches them through the CUDA driver API.

    python oracle/ref_cuda_build.py <directory holding cctpy's final_code/>
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile
import types

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
META = os.path.join(OUT, "cctpy_cuda.json")
KERNEL = "track_multi_particle_beamline_for_magnet_with_multi_qs"
# (name, cctpy float type, block_dim_x, max_current_element_number or None for cctpy's
# default): the speed test's FLOAT32 x 1024, the FLOAT64 block size cctpy's docstring asks for
# (1024 may exceed the register file in FP64), and both sized for gantry designs
CONFIGS = (("f32", "FLOAT32", 1024, None), ("f64", "FLOAT64", 512, None), ("f32_700k", "FLOAT32", 1024, 700_000),
           ("f64_700k", "FLOAT64", 512, 700_000))


def _stub_plotting():
    """Every cctpy package module imports pyplot at top level; tracking never calls it."""
    class _Any:
        def __getattr__(self, k):
            return _Any()

        def __call__(self, *a, **k):
            return _Any()

    for name in ("matplotlib", "matplotlib.pyplot", "mpl_toolkits", "mpl_toolkits.mplot3d"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    sys.modules["mpl_toolkits"].mplot3d = sys.modules["mpl_toolkits.mplot3d"]
    sys.modules["mpl_toolkits.mplot3d"].Axes3D = _Any


def cuda_sources(ref_dir: str) -> dict:
    """{name: (source, block_dim_x, max_current_element_number, max_qs_datas_length)} from
    cctpy's GPU_ACCELERATOR, in its CPU mode (no pycuda here) with its default capacities."""
    _stub_plotting()
    sys.path.insert(0, os.path.join(ref_dir, "final_code"))
    from packages.gpu_accelerator import GPU_ACCELERATOR
    out = {}
    for name, ftype, block, max_ce in CONFIGS:
        kw = {} if max_ce is None else {"max_current_element_number": max_ce}
        ga = GPU_ACCELERATOR(float_number_type=getattr(GPU_ACCELERATOR, ftype), block_dim_x=block, cpu_mode=True,
                             **kw)
        out[name] = (ga.cuda_code, ga.block_dim_x, ga.max_current_element_number, ga.max_qs_datas_length)
    return out


def build(ref_dir: str, nvcc: str = "nvcc", force: bool = False) -> dict:
    """Compile both configurations (skipped when the cubins of this exact source are there)."""
    src_file = os.path.join(ref_dir, "final_code", "packages", "gpu_accelerator.py")
    if not os.path.isfile(src_file):
        raise FileNotFoundError(f"no cctpy GPU module at {src_file}")
    with open(src_file, "rb") as f:
        sha = hashlib.sha256(f.read()).hexdigest()
    if not force and os.path.isfile(META):
        with open(META) as f:
            old = json.load(f)
        if old.get("source_sha256") == sha and all(
                os.path.isfile(os.path.join(OUT, c["cubin"])) for c in old.get("configs", {}).values()) \
                and set(old.get("configs", {})) == {c[0] for c in CONFIGS}:
            return old
    os.makedirs(OUT, exist_ok=True)
    meta = {"kernel": KERNEL, "source": "final_code/packages/gpu_accelerator.py", "source_sha256": sha,
            "arch": "sm_103a", "configs": {}}
    with tempfile.TemporaryDirectory() as tmp:
        ftypes = {c[0]: c[1] for c in CONFIGS}
        for name, (code, block, max_ce, max_qs) in cuda_sources(ref_dir).items():
            ftype = ftypes[name]
            cu = os.path.join(tmp, f"cctpy_{name}.cu")
            with open(cu, "w") as f:      # pycuda's SourceModule wraps the source the same way
                f.write('extern "C" {\n' + code + "\n}\n")
            cubin = os.path.join(OUT, f"cctpy_track_{name}.cubin")
            cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-Xptxas", "-v", "-o", cubin, cu]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for cctpy's {name} kernels:\n{r.stderr[-2000:]}")
            regs = None
            lines = r.stderr.splitlines()
            for i, line in enumerate(lines):
                if f"Compiling entry function '{KERNEL}'" in line:
                    for nxt in lines[i + 1:i + 4]:
                        m = re.search(r"Used (\d+) registers", nxt)
                        if m:
                            regs = int(m.group(1))
                            break
            if regs is not None and regs * block > 65536:
                raise RuntimeError(f"cctpy's {name} kernel uses {regs} registers: {block} threads do not fit an SM")
            meta["configs"][name] = {"cubin": os.path.basename(cubin), "block": block,
                                     "max_current_element_number": max_ce, "max_qs_datas_length": max_qs,
                                     "registers": regs, "float_bytes": 8 if ftype == "FLOAT64" else 4}
    with open(META, "w") as f:
        json.dump(meta, f, indent=1)
    return meta


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    print(json.dumps(build(sys.argv[1]), indent=1))
