"""Device-resident design sets and the calls into libcctgpu.

A *design* is one beamline (or magnet) reduced to what the kernels read: its
CCT current elements in the global frame (FP64, concatenated over layers) and
its QS records.  A *design set* concatenates several designs with CSR offsets,
so that one tracking launch covers a whole optimisation population.  Segment
sets stay in HBM between calls (cached on the Python object); the FP32c packed
form is built on first use.  Torch provides device memory and the stream.
"""
from __future__ import annotations

import ctypes
import threading
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _lib

_F32C_CACHE_ATTR = "_cctgpu_design"


def _device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("cctpy_gb300 needs a CUDA device (GB300, sm_103a); none is visible")
    return torch.device("cuda", torch.cuda.current_device())


def _ptr(t) -> int:
    return 0 if t is None or t.numel() == 0 else t.data_ptr()


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _classify(m):
    """The kind of a magnet the kernels evaluate (this package's classes or any object with
    cctpy's attributes): 'cct' (winding segments), 'qs', 'q', 'lum' (LocalUniformMagnet),
    'uniform' (UniformMagnet) -- analytic records --, 'wire' (Wire, AGCCT_CONNECTOR: current
    elements).  Raises ValueError otherwise."""
    if hasattr(m, "winding_number") and hasattr(m, "tilt_angles") and hasattr(m, "local_coordinate_system"):
        return "cct"
    if hasattr(m, "second_gradient") and hasattr(m, "aperture_radius") and hasattr(m, "local_coordinate_system"):
        return "qs"
    if hasattr(m, "magnetic_field") and hasattr(m, "aperture_radius") and hasattr(m, "local_coordinate_system"):
        return "lum"
    if hasattr(m, "gradient") and hasattr(m, "aperture_radius") and hasattr(m, "local_coordinate_system"):
        return "q"
    if hasattr(m, "elementary_current") and hasattr(m, "elementary_current_position") and hasattr(m, "current"):
        return "wire"
    if hasattr(m, "magnetic_field") and hasattr(getattr(m, "magnetic_field"), "x"):
        return "uniform"
    raise ValueError(f"magnet {m} cannot be evaluated on the GPU (CCT, QS, Q, LocalUniformMagnet, UniformMagnet, "
                     "Wire and AGCCT_CONNECTOR are supported)")


def magnet_list(obj) -> List:
    """Flatten a Beamline / CombinedMagnet / magnet (ours or cctpy's) into CCT/QS magnets."""
    if hasattr(obj, "magnets_for_gpu"):
        return obj.magnets_for_gpu()
    if hasattr(obj, "magnets"):               # cctpy Beamline
        out = []
        for m in obj.magnets:
            out.extend(magnet_list(m))
        return out
    if hasattr(obj, "get_magnets"):           # cctpy CombinedMagnet
        out = []
        for m in obj.get_magnets():
            out.extend(magnet_list(m))
        return out
    return [obj]


def cct_global_segments(m):
    """(kl, p0) global (N, 3) FP64 of a CCT (ours: vectorised; cctpy's: its own export)."""
    if hasattr(m, "global_segments"):
        return m.global_segments()
    kl, p0 = m.global_current_elements_and_elementary_current_positions(np.float64)
    return kl.reshape(-1, 3), p0.reshape(-1, 3)


def qs_record(m) -> np.ndarray:
    return np.asarray(m.to_numpy_array(np.float64), dtype=np.float64)


def _frame12(lcs) -> List[float]:
    return _xyz(lcs.location) + _xyz(lcs.XI) + _xyz(lcs.YI) + _xyz(lcs.ZI)


def analytic_record(m) -> Optional[np.ndarray]:
    """16-double record of an analytic magnet, or None if it contributes no field.
    QS: QS.to_numpy_array (magnets.py:726-748).  Q: the same with no sextupole term
    (magnets.py:762-801).  LocalUniformMagnet: frame, -length, field, 0, aperture (a negative
    length marks the uniform-field kind; magnets.py:440-481).  UniformMagnet: a frame whose YI
    is the field direction, length -inf (everywhere), |B| (magnets.py:417-437)."""
    kind = _classify(m)
    if kind == "qs":
        return qs_record(m)
    if kind == "q":
        return np.array(_frame12(m.local_coordinate_system) + [m.length, m.gradient, 0.0, m.aperture_radius])
    if kind == "lum":
        if not m.length > 0:
            return None
        return np.array(_frame12(m.local_coordinate_system) + [-float(m.length), float(m.magnetic_field), 0.0,
                                                                 float(m.aperture_radius)])
    if kind == "uniform":
        b = np.array(_xyz(m.magnetic_field))
        n = float(np.sqrt(b @ b))
        if n == 0.0:
            return None
        y = b / n
        helper = np.array([1.0, 0.0, 0.0]) if abs(y[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
        x = np.cross(y, helper)
        x /= np.sqrt(x @ x)
        z = np.cross(x, y)
        return np.concatenate([[0.0, 0.0, 0.0], x, y, z, [-np.inf, n, 0.0, np.inf]])
    raise ValueError(f"{m} is not an analytic magnet")


def wire_segments(m) -> Optional[tuple]:
    """(kl, p0) global (N, 3) current elements of a Wire (global path, cct.py:625-691) or an
    AGCCT_CONNECTOR (local path, moved to the global frame; cct.py:835-994), or None if it
    carries no current."""
    if approx_zero(float(m.current)):
        return None
    if hasattr(m, "start") and hasattr(m, "end") and not hasattr(m, "local_coordinate_system"):
        if _approx_equal(float(m.start), float(m.end)):
            return None
    kl = np.asarray(m.elementary_current, dtype=np.float64).reshape(-1, 3)
    p0 = np.asarray(m.elementary_current_position, dtype=np.float64).reshape(-1, 3)
    lcs = getattr(m, "local_coordinate_system", None)
    if lcs is not None:
        R = np.array([_xyz(lcs.XI), _xyz(lcs.YI), _xyz(lcs.ZI)])
        o = np.array(_xyz(lcs.location))
        kl = kl @ R
        p0 = o + p0 @ R
    return np.ascontiguousarray(kl), np.ascontiguousarray(p0)


def _approx_equal(a: float, b: float, err: float = 1e-6) -> bool:
    return a == b or abs(a - b) <= err or ((a + b != 0.0) and 2 * abs((a - b) / (a + b)) <= err)


def approx_zero(v: float) -> bool:
    return _approx_equal(v, 0.0)


LAYER_DOUBLES, LAYER_MAX_TILTS, LAYER_PARAMS = 32, 8, 10


def _xyz(p) -> List[float]:
    return [float(p.x), float(p.y), float(p.z)]


def layer_record(m, first: int = 0) -> np.ndarray:
    """The 32-double layer record of a CCT (ours or cctpy's) that cct_segments_build reads:
    frame (origin, XI, YI, ZI), big_r, small_r, current, xi/phi start and end, winding number,
    segments per winding, tilt count, tilt angles (degrees), index of its first segment."""
    lcs = m.local_coordinate_system
    tilts = [float(t) for t in m.tilt_angles]
    if len(tilts) > LAYER_MAX_TILTS:
        raise ValueError(f"{len(tilts)} tilt angles; the device generator takes at most {LAYER_MAX_TILTS}")
    s, e = m.starting_point_in_ksi_phi_coordinate, m.end_point_in_ksi_phi_coordinate
    r = np.zeros(LAYER_DOUBLES)
    r[0:12] = _xyz(lcs.location) + _xyz(lcs.XI) + _xyz(lcs.YI) + _xyz(lcs.ZI)
    r[12:22] = [m.big_r, m.small_r, m.current, s.x, s.y, e.x, e.y, m.winding_number,
                m.disperse_number_per_winding, len(tilts)]
    r[22:22 + len(tilts)] = tilts
    r[30] = first
    return r


def device_layers(magnets: Sequence) -> tuple:
    """(layer records, CCT magnets, analytic records (m, 16), other current elements (kl, p0)
    or None) of one design, with the CCT layers in host_design's order (zero-current layers
    dropped)."""
    recs, ccts, ana, wires = [], [], [], []
    for m in magnets:
        kind = _classify(m)
        if kind == "cct":
            if abs(float(m.current)) <= 1e-6:
                continue
            recs.append(layer_record(m))
            ccts.append(m)
        elif kind == "wire":
            w = wire_segments(m)
            if w is not None:
                wires.append(w)
        else:
            r = analytic_record(m)
            if r is not None:
                ana.append(r)
    extra = (np.concatenate([w[0] for w in wires]), np.concatenate([w[1] for w in wires])) if wires else None
    return recs, ccts, (np.stack(ana) if ana else np.zeros((0, 16))), extra


def host_design(magnets: Sequence) -> tuple:
    """(kls (N,3), p0s (N,3), analytic records (M,16)) of one design: the CCT layers' segments
    in magnet order, then the current elements of wires and connectors.  A CCT with
    |current| <= 1e-6 contributes nothing (cct.py:254-255)."""
    kls, p0s, ana, wkl, wp0 = [], [], [], [], []
    for m in magnets:
        kind = _classify(m)
        if kind == "cct":
            if abs(float(m.current)) <= 1e-6:
                continue
            kl, p0 = cct_global_segments(m)
            kls.append(kl)
            p0s.append(p0)
        elif kind == "wire":
            w = wire_segments(m)
            if w is not None:
                wkl.append(w[0])
                wp0.append(w[1])
        else:
            r = analytic_record(m)
            if r is not None:
                ana.append(r)
    kls += wkl
    p0s += wp0
    kl = np.concatenate(kls) if kls else np.zeros((0, 3))
    p0 = np.concatenate(p0s) if p0s else np.zeros((0, 3))
    qs = np.stack(ana) if ana else np.zeros((0, 16))
    return np.ascontiguousarray(kl), np.ascontiguousarray(p0), np.ascontiguousarray(qs)


class DesignSet:
    """Several designs resident in HBM: segments (FP64), QS records, CSR offsets.

    Built from host segment arrays (`designs`: per design (kls, p0s, qs)) or, with
    `DesignSet.from_layers`, from CCT layer records with the segments generated on the
    device (cct_segments_build); the latter keeps the records (`layers`, `h_layers`) and
    each layer's design (`layer_design`) for the parameter Jacobian."""

    def __init__(self, designs: Sequence[tuple]):
        seg_counts = [d[0].shape[0] for d in designs]
        # a design given several times (the same tuple object) is copied to the device once
        # and repeated there
        first = {}
        order = [first.setdefault(id(d), len(first)) for d in designs]
        uniq = [None] * len(first)
        for d, i in zip(designs, order):
            uniq[i] = d
        cat = lambda k, w: np.concatenate([d[k] for d in uniq]) if uniq else np.zeros((0, w))
        dev = _device()
        kls, p0s = torch.from_numpy(cat(0, 3)).to(dev), torch.from_numpy(cat(1, 3)).to(dev)
        if len(uniq) < len(designs):
            off = np.concatenate([[0], np.cumsum([d[0].shape[0] for d in uniq])]).astype(np.int64)
            kls = torch.cat([kls[off[i]:off[i + 1]] for i in order])
            p0s = torch.cat([p0s[off[i]:off[i + 1]] for i in order])
        self._finish(seg_counts, [d[2] for d in designs], kls, p0s)

    def _finish(self, seg_counts, qs_list, kls, p0s):
        dev = kls.device
        self.n_designs = len(seg_counts)
        if self.n_designs == 0:
            raise ValueError("empty design set")
        self.h_seg_off = np.concatenate([[0], np.cumsum(seg_counts)]).astype(np.int64)
        self.h_qs_off = np.concatenate([[0], np.cumsum([q.shape[0] for q in qs_list])]).astype(np.int64)
        self.kls, self.p0s = kls, p0s
        qs = np.concatenate(qs_list) if qs_list else np.zeros((0, 16))
        self.qs = torch.from_numpy(np.ascontiguousarray(qs, dtype=np.float64).reshape(-1, 16)).to(dev)
        self.seg_off = torch.from_numpy(self.h_seg_off).to(dev)
        self.qs_off = torch.from_numpy(self.h_qs_off).to(dev)
        self._packed = None
        if not hasattr(self, "layers"):
            self.layers = self.h_layers = self.layer_design = None

    @classmethod
    def from_layers(cls, layer_lists: Sequence[Sequence[np.ndarray]], qs_lists: Sequence[np.ndarray],
                    extra_segments: Sequence = None) -> "DesignSet":
        """Design set whose CCT segments are generated on the device from layer records
        (`layer_record`): layer_lists[d] = records of design d, qs_lists[d] = (m, 16) analytic
        records, extra_segments[d] = None or (kl, p0) global current elements of the design's
        wires and connectors (placed after its layers)."""
        lib = _lib.load()
        dev = _device()
        self = cls.__new__(cls)
        extra = extra_segments or [None] * len(layer_lists)
        recs, seg_counts, at = [], [], 0
        self.layer_design = []
        for d, ls in enumerate(layer_lists):
            start = at
            for r in ls:                                   # layers first, in order
                r = np.array(r, dtype=np.float64)
                r[30] = at
                recs.append(r)
                self.layer_design.append(d)
                at += int(r[19]) * int(r[20])
            if extra[d] is not None:                       # then the design's other current elements
                at += int(extra[d][0].shape[0])
            seg_counts.append(at - start)
        self.layer_design = np.array(self.layer_design, dtype=np.int64)
        self.h_layers = np.ascontiguousarray(np.stack(recs) if recs else np.zeros((0, LAYER_DOUBLES)))
        n = at
        if recs:
            total = lib.cct_layer_segments(self.h_layers.ctypes.data_as(ctypes.c_void_p), len(recs))
            _lib.check(0 if total >= 0 else _lib.CCT_ERR_ARG, "cct_layer_segments")
        kls = torch.empty((n, 3), dtype=torch.float64, device=dev)
        p0s = torch.empty((n, 3), dtype=torch.float64, device=dev)
        self.layers = torch.from_numpy(self.h_layers).to(dev)
        if recs:
            _lib.check(lib.cct_segments_build(_ptr(self.layers), len(recs), _ptr(kls), _ptr(p0s), n, _stream()),
                       "cct_segments_build")
        at = 0
        for d, ls in enumerate(layer_lists):
            at += sum(int(r[19]) * int(r[20]) for r in ls)
            if extra[d] is not None:
                k = int(extra[d][0].shape[0])
                kls[at:at + k] = torch.as_tensor(extra[d][0], dtype=torch.float64, device=dev)
                p0s[at:at + k] = torch.as_tensor(extra[d][1], dtype=torch.float64, device=dev)
                at += k
        self._finish(seg_counts, [np.asarray(q, dtype=np.float64).reshape(-1, 16) for q in qs_lists], kls, p0s)
        return self

    def param_grad(self, seg_grad: torch.Tensor) -> np.ndarray:
        """(n_layers, 10) dJ/d(tilt 0..7 [deg], current [A], big_r [m]) of every layer from a
        device segment gradient (n_segments, 6) (cct_segments_param_grad)."""
        if self.layers is None:
            raise ValueError("param_grad needs a design set built from layer records (DesignSet.from_layers)")
        lib = _lib.load()
        g = seg_grad.to(dtype=torch.float64).contiguous()
        if g.shape != (self.n_segments, 6) or not g.is_cuda:
            raise ValueError(f"segment gradient must be a CUDA (n_segments, 6) tensor, not {tuple(g.shape)}")
        out = torch.empty((self.h_layers.shape[0], LAYER_PARAMS), dtype=torch.float64, device=g.device)
        _lib.check(lib.cct_segments_param_grad(_ptr(self.layers), self.h_layers.shape[0], _ptr(g), self.n_segments,
                                               _ptr(out), _stream()), "cct_segments_param_grad")
        return out.cpu().numpy()

    @property
    def n_segments(self) -> int:
        return int(self.h_seg_off[-1])

    def segments_of(self, d: int) -> int:
        return int(self.h_seg_off[d + 1] - self.h_seg_off[d])

    def packed(self) -> torch.Tensor:
        """FP32c packed tiles (built once, on the current stream)."""
        if self._packed is None:
            lib = _lib.load()
            off = self.h_seg_off.ctypes.data_as(ctypes.c_void_p)
            nbytes = lib.cct_f32c_packed_bytes(off, self.n_designs)
            _lib.check(0 if nbytes >= 0 else _lib.CCT_ERR_ARG, "cct_f32c_packed_bytes")
            buf = torch.empty(int(nbytes) + 256, dtype=torch.uint8, device=self.kls.device)
            shift = (-buf.data_ptr()) % 256
            view = buf[shift:shift + int(nbytes)]
            _lib.check(lib.cct_f32c_pack(_ptr(self.kls), _ptr(self.p0s), off, self.n_designs, view.data_ptr(),
                                         int(nbytes), _stream()), "cct_f32c_pack")
            self._packed_buf = buf
            self._packed = view
        return self._packed


def design_of(obj) -> DesignSet:
    """Single-design set of a magnet / beamline, cached on the object."""
    ds = getattr(obj, _F32C_CACHE_ATTR, None)
    if ds is None:
        ds = DesignSet([host_design(magnet_list(obj))])
        try:
            setattr(obj, _F32C_CACHE_ATTR, ds)
        except AttributeError:
            pass
    return ds


def design_set_of(objs: Sequence, segments: str = "host") -> DesignSet:
    """Design set of several beamlines / magnets.  segments="host" builds the segment arrays
    with numpy and copies them; "device" generates them on the GPU from layer records."""
    if segments == "host":
        built = {}
        for o in objs:      # an object given several times: built once, repeated on the device
            if id(o) not in built:
                built[id(o)] = host_design(magnet_list(o))
        return DesignSet([built[id(o)] for o in objs])
    if segments != "device":
        raise ValueError(f"segments must be 'host' or 'device', not {segments!r}")
    parts = [device_layers(magnet_list(o)) for o in objs]
    ds = DesignSet.from_layers([p[0] for p in parts], [p[2] for p in parts], [p[3] for p in parts])
    ds.layer_magnets = [m for p in parts for m in p[1]]
    return ds


def field_at_points(ds: DesignSet, points, precision: str = "f64", design: int = 0, out_host=None):
    """Field of design `design` at (n, 3) points.

    points: numpy array (-> numpy result), torch CUDA tensor (-> CUDA tensor, no copies) or
    torch CPU tensor (-> CPU tensor; pinned memory gives asynchronous copies; `out_host`,
    a CPU float64 tensor of the same shape, receives the result without an allocation)."""
    lib = _lib.load()
    dev = ds.kls.device
    if not 0 <= design < ds.n_designs:
        raise ValueError(f"design {design} not in a set of {ds.n_designs}")
    as_numpy = not isinstance(points, torch.Tensor)
    host_tensor = (not as_numpy) and not points.is_cuda
    if as_numpy:
        pts = torch.as_tensor(np.ascontiguousarray(points, dtype=np.float64), device=dev)
    elif host_tensor:
        pts = points.to(device=dev, dtype=torch.float64, non_blocking=True).contiguous()
    else:
        pts = points.to(dtype=torch.float64).contiguous()
    if pts.ndim != 2 or pts.shape[1] != 3:
        raise ValueError(f"points must have shape (n, 3), not {tuple(pts.shape)}")
    out = torch.empty_like(pts)
    a, b = int(ds.h_seg_off[design]), int(ds.h_seg_off[design + 1])
    qa, qb = int(ds.h_qs_off[design]), int(ds.h_qs_off[design + 1])
    qs = ds.qs[qa:qb]
    if precision == "f64":
        kls, p0s = ds.kls[a:b], ds.p0s[a:b]
        rc = lib.cct_field_f64(_ptr(kls), _ptr(p0s), b - a, _ptr(qs), qb - qa, _ptr(pts), pts.shape[0], _ptr(out),
                               _stream())
        _lib.check(rc, "cct_field_f64")
    elif precision == "f32c":
        rc = lib.cct_field_f32c(ds.packed().data_ptr(), design, _ptr(qs), qb - qa, _ptr(pts), pts.shape[0],
                                _ptr(out), _stream())
        _lib.check(rc, "cct_field_f32c")
    else:
        raise ValueError(f"precision must be 'f64' or 'f32c', not {precision!r}")
    if as_numpy:
        return out.cpu().numpy()
    if host_tensor:
        res = out_host if out_host is not None else torch.empty(out.shape, dtype=torch.float64,
                                                                 pin_memory=points.is_pinned())
        res.copy_(out, non_blocking=res.is_pinned())
        torch.cuda.current_stream().synchronize()
        return res
    return out


def field_status() -> None:
    """Raise if an FP32c field call on this device (any stream) since the last check was given
    a buffer that is not a packed set or a design it does not hold (ValueError), or gave up
    waiting for a tile copy (CctTimeoutError); the fields of such a call are NaN.  Clears the
    status; waits for the current stream (cct_field_status)."""
    _device()
    _lib.check(_lib.load().cct_field_status(_stream()), "cct_field_status")


_scratch_cache = {}
# One scratch buffer per device, shared by the synchronous calls below: ctypes releases the GIL
# during a library call, so calls from several host threads take this lock around its use.
_scratch_lock = threading.Lock()


def scratch(nbytes: int, dev) -> torch.Tensor:
    """The device's shared 256-byte-aligned scratch of at least nbytes (hold _scratch_lock)."""
    key = (dev.index,)
    buf = _scratch_cache.get(key)
    if buf is None or buf.numel() < nbytes + 256:
        buf = torch.empty(int(nbytes) + 256, dtype=torch.uint8, device=dev)
        _scratch_cache[key] = buf
    shift = (-buf.data_ptr()) % 256
    return buf[shift:shift + int(nbytes)]


def track(ds: DesignSet, particles, distance: float, footstep: float, precision: str = "f64"):
    """RK4-track particle records through every design of `ds`.

    particles: (n_designs, n_p, 10) or (n_p, 10) (broadcast to every design) FP64 records,
    numpy or torch CUDA.  Returns (n_designs, n_p, 10) in the same kind."""
    lib = _lib.load()
    dev = ds.kls.device
    as_numpy = not isinstance(particles, torch.Tensor)
    p = torch.as_tensor(np.asarray(particles, dtype=np.float64) if as_numpy else particles, dtype=torch.float64,
                        device=dev)
    if p.ndim == 2:
        p = p.unsqueeze(0).expand(ds.n_designs, -1, -1)
    if p.ndim != 3 or p.shape[0] != ds.n_designs or p.shape[2] != 10:
        raise ValueError(f"particles must be (n_designs, n, 10) or (n, 10), not {tuple(p.shape)}")
    p = p.contiguous().clone()
    n_p = p.shape[1]
    if n_p == 0:
        return p.cpu().numpy() if as_numpy else p
    prec = {"f64": 0, "f32c": 1}.get(precision)
    if prec is None:
        raise ValueError(f"precision must be 'f64' or 'f32c', not {precision!r}")
    packed = ds.packed() if prec == 1 else None
    nbytes = lib.cct_track_scratch_bytes(ds.n_designs, n_p)
    _lib.check(0 if nbytes >= 0 else _lib.CCT_ERR_ARG, "cct_track_scratch_bytes")
    with _scratch_lock:
        sc = scratch(nbytes, dev)
        rc = lib.cct_track(_ptr(ds.kls), _ptr(ds.p0s), _ptr(ds.seg_off), 0 if packed is None else packed.data_ptr(),
                           _ptr(ds.qs), _ptr(ds.qs_off), ds.n_designs, _ptr(p), n_p, float(distance),
                           float(footstep), prec, sc.data_ptr(), int(nbytes), _stream())
    _lib.check(rc, "cct_track")
    return p.cpu().numpy() if as_numpy else p


def _track_args(ds: DesignSet, precision: str):
    prec = {"f64": 0, "f32c": 1}.get(precision)
    if prec is None:
        raise ValueError(f"precision must be 'f64' or 'f32c', not {precision!r}")
    packed = ds.packed().data_ptr() if prec == 1 else 0
    return prec, packed


class TrackLaunch:
    """cct_track_async on device buffers that stay in place, so that the launch can be
    captured in a CUDA graph (torch.cuda.graph) and replayed: `particles` is a CUDA tensor
    (n_designs, n, 10) tracked in place; call status() after the launch (or the replay) has
    been enqueued to synchronise and raise on an error."""

    def __init__(self, ds: DesignSet, particles: torch.Tensor, distance: float, footstep: float,
                 precision: str = "f32c"):
        if not (isinstance(particles, torch.Tensor) and particles.is_cuda and particles.dtype == torch.float64
                and particles.ndim == 3 and particles.shape[0] == ds.n_designs and particles.shape[2] == 10
                and particles.is_contiguous()):
            raise ValueError("particles must be a contiguous CUDA float64 tensor (n_designs, n, 10)")
        self.ds, self.particles = ds, particles
        self.distance, self.footstep = float(distance), float(footstep)
        self.prec, self.packed = _track_args(ds, precision)
        lib = _lib.load()
        n = lib.cct_track_scratch_bytes(ds.n_designs, particles.shape[1])
        _lib.check(0 if n >= 0 else _lib.CCT_ERR_ARG, "cct_track_scratch_bytes")
        self._buf = torch.empty(int(n) + 256, dtype=torch.uint8, device=particles.device)
        shift = (-self._buf.data_ptr()) % 256
        self.scratch = self._buf[shift:shift + int(n)]

    def launch(self) -> None:
        lib = _lib.load()
        ds = self.ds
        rc = lib.cct_track_async(_ptr(ds.kls), _ptr(ds.p0s), _ptr(ds.seg_off), self.packed, _ptr(ds.qs),
                                 _ptr(ds.qs_off), ds.n_designs, self.particles.data_ptr(), self.particles.shape[1],
                                 self.distance, self.footstep, self.prec, self.scratch.data_ptr(),
                                 self.scratch.numel(), _stream())
        _lib.check(rc, "cct_track_async")

    def status(self) -> None:
        _lib.check(_lib.load().cct_track_status(self.scratch.data_ptr(), _stream()), "cct_track_status")


def autotune(ds: DesignSet, particles, footstep: float, precision: str = "f32c", steps: int = 4) -> int:
    """Time `steps` RK4 steps of this problem for several work splits -- the FP32c particle
    block (particles a unit sums for together) and the units of design x particle block x
    segment chunk per CTA --, keep the fastest for later tracking calls of the process and
    return its units per CTA (cct_autotune; `particle_block()` gives its particle block)."""
    lib = _lib.load()
    dev = ds.kls.device
    p = torch.as_tensor(np.asarray(particles, dtype=np.float64) if not isinstance(particles, torch.Tensor)
                        else particles, dtype=torch.float64, device=dev)
    if p.ndim == 2:
        p = p.unsqueeze(0).expand(ds.n_designs, -1, -1)
    p = p.contiguous()
    prec, packed = _track_args(ds, precision)
    n = lib.cct_autotune_scratch_bytes(ds.n_designs, p.shape[1])
    _lib.check(0 if n >= 0 else _lib.CCT_ERR_ARG, "cct_autotune_scratch_bytes")
    best = ctypes.c_int32(0)
    with _scratch_lock:
        sc = scratch(int(n), dev)
        rc = lib.cct_autotune(_ptr(ds.kls), _ptr(ds.p0s), _ptr(ds.seg_off), packed, _ptr(ds.qs), _ptr(ds.qs_off),
                              ds.n_designs, p.data_ptr(), p.shape[1], float(footstep), prec, int(steps),
                              sc.data_ptr(), int(n), ctypes.byref(best), _stream())
    _lib.check(rc, "cct_autotune")
    return int(best.value)


def set_units_per_cta(n: int = 0) -> None:
    """Set the tracking work split by hand (0 restores the default of 8)."""
    _lib.check(_lib.load().cct_track_set_units_per_cta(int(n)), "cct_track_set_units_per_cta")


def set_particle_block(n: int = 0) -> None:
    """Set the FP32c particle block by hand: 16, 32, 64, 128 or 256 (0 restores the automatic
    choice)."""
    _lib.check(_lib.load().cct_track_set_particle_block(int(n)), "cct_track_set_particle_block")


def particle_block() -> int:
    """The process-wide FP32c particle block (0: automatic)."""
    return int(_lib.load().cct_track_particle_block())
