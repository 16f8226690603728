"""Split-precision form of the PIC step (``SplitRun``).

The precision pattern of the GB300 build: particles in FP32 with the x
position stored as an int32 cell index plus an FP32 offset, complex64
fields, the DHT / mode-coupling products on the tcgen05 tensor cores as
3-term split-BF16 products with FP32 accumulation.  FP64 is kept for the
operator build (Bessel-zero DHT matrices, PSATD coefficients), for the
running window origin ``leftX`` and for the initial half step.

``SplitRun(SimComps)`` takes the same components as ``ChimeraRun``; it first
builds the FP64 ``ChimeraRun`` (which performs the reference's initial half
step), converts its state, and then advances every ``make_step(istep)`` with
the split kernels.  ``to_fp64()`` writes the state back into the solver's and
species' FP64 ``Data`` for diagnostics.

Supported: plain (non-envelope) solver, SpaceCharge, StillAsBackground,
NoPoissonCorrection, Still species, moving window with AbsorbLayer /
AddPlasma / IonsOnTop / Staged.  Not in this form (raises): the envelope
(KxShift) solver, devices, StaticKick.  Deposits follow the serial
``dep_curr`` / ``dep_dens`` semantics (the chunked variants only differ by
the dropped x-node-0 contributions of chunk 0 and by summation order).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from . import fimera as chimera
from .chimera_main import ChimeraRun


class SpOps(C.Structure):
    _fields_ = [("K", C.c_int32), ("N", C.c_int32), ("nmodes", C.c_int32), ("pad", C.c_int32),
                ("f32", C.c_void_p), ("bf16", C.c_void_p * 3)]


def _prepare_ops(mats: np.ndarray, device) -> tuple:
    """FP64 (K, N, nmodes) Fortran-ordered matrices -> prepared operator set."""
    K, N, nm = mats.shape
    d = torch.from_numpy(np.asfortranarray(mats, dtype=np.float64)).to(device)
    buf = torch.empty(_lib.query("chm_sp_ops_bytes", K, N, nm), dtype=torch.uint8, device=device)
    ops = SpOps()
    _lib.call("chm_sp_prepare_ops", C.addressof(ops), d.data_ptr(), K, N, nm, buf.data_ptr(),
              buf.numel(), torch.cuda.current_stream().cuda_stream)
    return ops, buf, d


def _c64(t: torch.Tensor) -> torch.Tensor:
    """complex128 Fortran tensor -> complex64 Fortran tensor."""
    out = chimera.fortran_empty(tuple(t.shape), dtype=torch.complex64, device=t.device)
    out.copy_(t)
    return out


def _f32(a, device) -> torch.Tensor:
    arr = np.asfortranarray(np.asarray(a), dtype=np.float32)
    return torch.from_numpy(arr).to(device)


def _slots(n: int) -> int:
    """Slots of the tile layout holding n particles (whole tiles of 512)."""
    return (int(n) + 511) // 512 * 512


def cell_order(coords, X0: float, dx: float, dr: float, patch: int = 4):
    """Stable permutation of particles into deposit order: patches of
    patch x patch generation cells (cells [X0 + i dx, X0 + (i+1) dx) x
    [j dr, (j+1) dr)), patch rows in a serpentine order (so consecutive
    patches are neighbours), the cells of a patch in serpentine order too,
    and within a cell its two deposit cells (r nodes at (j - 1/2) dr) in
    turn.  A block of particles then covers a compact patch of the grid (a
    small deposit box), and the runs of 16 consecutive particles of the tile
    layout share a deposit cell.  coords: (3, n) numpy or torch array."""
    lib = torch if isinstance(coords, torch.Tensor) else np
    x, y, z = coords[0], coords[1], coords[2]
    n = x.shape[0]
    if n == 0:
        return torch.arange(0, device=x.device) if lib is torch else np.arange(0)
    s = lib.sqrt(y * y + z * z) / dr
    gx = lib.floor((x - X0) / dx)
    gr = lib.floor(s)
    half = (s - gr >= 0.5)  # upper deposit cell of the generation cell
    if lib is torch:
        gx, gr, half = gx.to(torch.int64), gr.to(torch.int64).clamp(min=0), half.to(torch.int64)
    else:
        gx, gr, half = gx.astype(np.int64), np.maximum(gr.astype(np.int64), 0), half.astype(np.int64)
    gx = gx - gx.min()
    P = int(patch)
    px, lx = gx // P, gx % P
    pr, lr = gr // P, gr % P
    # patch columns: the exact count on the host; on the device a fixed bound
    # (the order is the same, and no device-to-host read stalls the stream)
    npx = int(px.max()) + 1 if lib is np else 1 << 20
    px = lib.where(pr % 2 == 1, npx - 1 - px, px)  # serpentine patch rows
    lx = lib.where(lr % 2 == 1, P - 1 - lx, lx)    # serpentine rows in a patch
    key = (((pr * npx + px) * P + lr) * P + lx) * 2 + half
    if lib is torch:
        return torch.argsort(key, stable=True)
    return np.argsort(key, kind="stable")


class _SpParticles:
    """Split-layout SoA buffers of one species (tile layout, see
    chm_sp_slot; whole tiles allocated with spare capacity).

    Absorbed particles stay in place, marked in ``dead`` with zero weight,
    until ``compact`` drops them; ``counters`` (device) holds the number of
    dead particles and the running sum of live particles over steps."""

    NAMES = ("ix", "fx", "y", "z", "px", "py", "pz", "w")

    def __init__(self, device, cap):
        self.device = device
        self.cap = 0
        self.n = 0
        self.buf = {}
        self.spare = None
        self.dead = None
        self.counters = torch.zeros(2, dtype=torch.int64, device=device)
        self.moves = 0  # window moves since the last compaction
        self.reserve(cap)

    def _alloc(self, cap):
        return {k: torch.zeros(cap, dtype=torch.int32 if k == "ix" else torch.float32,
                               device=self.device) for k in self.NAMES}

    def reserve(self, cap):
        cap = _slots(max(cap, 1024))
        if cap <= self.cap:
            return
        new = self._alloc(cap)
        dead = torch.zeros(cap, dtype=torch.uint8, device=self.device)
        if self.n:
            used = _slots(self.n)  # whole tiles keep the slot of every particle
            for k in self.NAMES:
                new[k][:used].copy_(self.buf[k][:used])
            dead[:used].copy_(self.dead[:used])
        self.buf, self.dead, self.cap = new, dead, cap
        self.spare = None

    def ptrs(self, buf=None):
        b = self.buf if buf is None else buf
        return [b[k].data_ptr() for k in self.NAMES]

    def append_f64(self, coords, momenta, weights, X0, dx):
        m = int(coords.shape[-1])
        if m == 0:
            return
        if _slots(self.n + m) > self.cap:
            self.reserve(max(self.n + m, int(1.5 * self.cap)))
        dev = self.device
        if all(isinstance(a, torch.Tensor) and a.device.type == "cuda"
               for a in (coords, momenta, weights)):
            tx, tp, tw = (t.to(torch.float64) for t in (coords, momenta, weights))
        else:
            # host arrays: one pinned staging buffer and one asynchronous copy
            # (a pageable copy would wait for the work queued on the stream)
            stage = torch.empty(7 * m, dtype=torch.float64, pin_memory=True)
            h = stage.numpy()
            for a, lo, nc in ((coords, 0, 3), (momenta, 3 * m, 3), (weights, 6 * m, 1)):
                src = a.cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
                h[lo:lo + nc * m].reshape(nc, m)[...] = src.reshape(nc, m)
            chimera.io_bytes["h2d"] += 7 * m * 8
            d = stage.to(dev, non_blocking=True)
            tx, tp, tw = d[:3 * m].view(3, m), d[3 * m:6 * m].view(3, m), d[6 * m:]
        _lib.call("chm_sp_from_f64", *self.ptrs(), self.dead.data_ptr(), self.n, tx.data_ptr(),
                  tx.stride(0), tx.stride(1), tp.data_ptr(), tp.stride(0), tp.stride(1),
                  tw.data_ptr(), tw.stride(0), float(X0), float(dx), m, _stream())
        self.n += m

    def sort_cells(self, win_k, win_f, nx, nr, dr_inv):
        """Re-sort the particles by deposit cell (chm_sp_sort_cells), dropping
        the dead ones; one device->host read (the live count)."""
        if self.n == 0:
            return
        if self.spare is None:
            self.spare = self._alloc(self.cap)
        ws = chimera.workspace(_lib.query("chm_sp_sort_ws_bytes", self.n), self.device)
        n_out = torch.empty(1, dtype=torch.int64, device=self.device)
        _lib.call("chm_sp_sort_cells", *self.ptrs(), self.dead.data_ptr(), self.n, int(win_k),
                  float(win_f), int(nx), int(nr), float(dr_inv), *self.ptrs(self.spare),
                  n_out.data_ptr(),
                  ws.data_ptr(), ws.numel(), _stream())
        n = int(n_out.item())
        chimera.io_bytes["d2h"] += 8
        self.buf, self.spare = self.spare, self.buf
        self.n = n
        self.dead[:_slots(n)].zero_()
        self.counters[0].zero_()
        self.moves = 0

    def compact(self):
        """Drop the dead particles (stable order); one device->host read."""
        if self.n == 0:
            return
        if self.spare is None:
            self.spare = self._alloc(self.cap)
        ws = chimera.workspace(_lib.query("chm_sp_compact_ws_bytes", self.n), self.device)
        n_out = torch.empty(1, dtype=torch.int64, device=self.device)
        _lib.call("chm_sp_compact", *self.ptrs(), self.dead.data_ptr(), self.n,
                  *self.ptrs(self.spare), n_out.data_ptr(), ws.data_ptr(), ws.numel(), _stream())
        n = int(n_out.item())
        chimera.io_bytes["d2h"] += 8
        self.buf, self.spare = self.spare, self.buf
        self.n = n
        self.dead[:_slots(n)].zero_()
        self.counters[0].zero_()
        self.moves = 0


def _stream():
    return torch.cuda.current_stream().cuda_stream


def window_cells(leftX, X0, dx):
    """The window's position in cells from X0, (k, fd): k = floor((leftX -
    X0) / dx) and the FP64 fraction fd, as chm_sp_window_set computes them."""
    sv = (float(leftX) - float(X0)) / float(dx)
    k = np.floor(sv)
    return int(k), float(sv - k)


def window_cells_after(k, fd, shift, dx):
    """(k, fd) after a window move by shift, as chm_sp_window_advance computes
    them: fd + shift / dx in FP64, its whole part carried into k (a move by a
    whole number of cells leaves fd exactly as it was)."""
    s = float(fd) + float(shift) / float(dx)
    fl = np.floor(s)
    return int(k) + int(fl), float(s - fl)


# device functions of fimera the split form fuses into its gather + push
# (chm_sp_gather_push_env und_kind)
_UNDULATORS = {"undul_analytic": 1, "undul_analytic_taper": 2, "undul_mapped": 3,
               "undul_mapped_tap": 4}
_UND_PARAMS = {1: 4, 2: 5, 3: 3, 4: 5}  # params(n) of devices.f90 per kind


def fused_undulator(devices, device):
    """The undulator of a species' Devices as the split push takes it:
    None, or (und_kind, params, map) with the map a0(2, nmap) as nmap FP32
    column pairs on `device` (None for the analytic kinds).  Raises for a
    device the split form does not fuse, for more than one device, and for
    a parameter array of the wrong length (f2py's dimension check,
    devices.f90:18-203)."""
    und = None
    for d in devices:
        kind = _UNDULATORS.get(getattr(d[0], "__name__", ""))
        if kind is None or und is not None or len(d) != (2 if kind <= 2 else 3):
            raise NotImplementedError(
                "the split form fuses one undulator (undul_analytic[_taper] or "
                "undul_mapped[_tap]) per species into the push")
        prm = np.asarray(d[-1], dtype=np.float64).ravel()
        if prm.size != _UND_PARAMS[kind]:
            raise ValueError(f"{d[0].__name__}: params has {prm.size} values, "
                             f"expected {_UND_PARAMS[kind]}")
        amap = None
        if kind >= 3:
            a = torch.as_tensor(d[1])
            if a.dim() != 2 or a.shape[0] != 2 or a.shape[1] < 1:
                raise ValueError(f"{d[0].__name__}: the map is a0(2, nmap)")
            amap = a.t().to(device=device, dtype=torch.float32).contiguous()
        und = (kind, prm, amap)
    return und


class SortCadence:
    """Run-time choice of the re-sort cadence (steps between two sorts by
    deposit cell).  As particles drift, the cell runs of the deposit and
    gather kernels break up and those kernels slow down by g per step; a
    sort costs a fixed time S and recovers what the drift cost.  Sorting
    every c steps then costs S / c + g c / 2 per step, least at
    c = sqrt(2 S / g).  S is timed directly; g is the time a sort recovers
    (the step time of the last steps before a sort minus that of the first
    steps after it) over the steps since the previous sort, so that the
    physical growth of the work (more particles moving as the laser enters
    the plasma) is not mistaken for disorder.  When a sort recovers nothing
    the cadence goes to its maximum.  The step times come from CUDA events
    read back at the next sort, so no step waits for them; ``history`` keeps
    (step, cadence, sort ms, recovered ms per step) for the record."""

    NAVG = 4  # steps averaged on each side of a sort

    def __init__(self, start=32, lo=8, hi=512):
        self.cadence, self.lo, self.hi = start, lo, hi
        self.history = []
        self._events = []      # (steps since sort, start, end) of the interval's steps
        self._sort_ev = None   # (start, end) of the last sort
        self._tail = None      # mean step ms of the last steps before the last sort
        self._last_len = None  # steps of the interval that ended with the last sort

    def step_events(self, since):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        self._events.append((since, a, b))
        return a, b

    def sort_events(self):
        self._sort_ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        return self._sort_ev

    def update(self, step):
        """After a sort (the stream has been synchronised by its count read)."""
        t = [v for _, v in sorted((s, a.elapsed_time(b)) for s, a, b in self._events
                                  if a.query() and b.query())]
        self._events = []
        S = self._sort_ev[0].elapsed_time(self._sort_ev[1]) if self._sort_ev else None
        g = None
        if len(t) >= 2 * self.NAVG:
            head = float(np.mean(t[:self.NAVG]))
            if self._tail is not None and self._last_len and S is not None:
                g = (self._tail - head) / self._last_len
                c = self.hi if g <= 0 else int(np.sqrt(2.0 * S / g))
                self.cadence = int(min(self.hi, max(self.lo, c)))
            self._tail = float(np.mean(t[-self.NAVG:]))
        self._last_len = len(t)
        self.history.append((int(step), int(self.cadence), S, g))


class SplitRun:
    """Precision form of ``ChimeraRun`` (same SimComps, same make_step)."""

    def __init__(self, SimComps, fp64_run: ChimeraRun | None = None):
        self.fp = fp64_run if fp64_run is not None else ChimeraRun(SimComps)
        if len(self.fp.Solvers) != 1:
            raise NotImplementedError("the split form runs one solver")
        self.solver = S = self.fp.Solvers[0]
        A = S.Args
        feats = A["Features"]
        if "StaticKick" in feats:
            raise NotImplementedError("the split form covers the time-stepped solvers")
        # envelope (KxShift) solver: modes -K..K, J_z deposit with the
        # carrier e^{-i kx0 x}, complex PSATD coefficients
        self.env = "KxShift" in A
        if self.env and ("SpaceCharge" in feats or "StillAsBackground" in feats):
            raise NotImplementedError("the envelope charge deposit is not in the split form")
        # external fields: the undulators, fused into the gather; a mapped
        # one carries its map a0(2, nmap) as FP32 column pairs on the device
        self.undulators = [fused_undulator(sp.Devices, S.device) for sp in self.fp.Particles]
        if any(self.undulators) and not self.env:
            raise NotImplementedError("the split form fuses undulators into the envelope push only")
        dev = self.device = S.device
        self.space_charge = "SpaceCharge" in feats
        self.poisson = "NoPoissonCorrection" not in feats
        self.nx, self.nr, self.nkr, self.nm = A["Nx"], A["Nr"], A["Nkr"], A["Mtot"]
        self.dx, self.dt = A["dx"], A["TimeStep"]
        self.X0 = float(A["Xgrid"][0])  # fixed origin of the particle cell index
        # the window origin on the device (chm_sp_window: leftX, X0, dx, k, f),
        # advanced on the stream at every window move, so the step's kernels
        # read the current origin also when the step replays as a CUDA graph
        self.win = torch.zeros(64, dtype=torch.uint8, device=S.device)
        self._win_set(float(A["leftX"]))
        # operators (FP64 host build -> FP32 copy + split BF16)
        self._keep = []
        self.ops = {}
        for name, key in (("InCurr", "InCurr"), ("Out", "Out"), ("Dp", "DpS2S"), ("Dm", "DmS2S")):
            ops, buf, d = _prepare_ops(A[key], dev)
            self.ops[name] = ops
            self._keep += [buf, d]
        # kx of the derivatives (kx0 + kx_env for the envelope solver) and of
        # the transforms' shift (kx_env for the envelope solver)
        self.kx64 = S.dev["kx"]
        self.kx32 = self.kx64.to(torch.float32)
        self.kxb64 = S.dev["kx_base"]
        self.depfact = _f32(A["DepFact"], dev)
        self.pf = _f32(A["PoissFact"], dev)
        CE, CG = S.Data["PSATD_E"], S.Data["PSATD_G"]
        self.complex_psatd = CE.is_complex()
        self.nterm = CE.shape[-1]
        cdt = torch.complex64 if self.complex_psatd else torch.float32
        self.c1 = chimera.fortran_empty(tuple(CE.shape), cdt, dev)
        self.c1.copy_(CE)
        self.c2 = chimera.fortran_empty(tuple(CG.shape), cdt, dev)
        self.c2.copy_(CG)
        if self.complex_psatd and (self.nterm != 3 or self.poisson):
            raise NotImplementedError("complex PSATD coefficients without space charge and "
                                      "without the Poisson correction")
        if self.env:
            # carrier table of the window's cells (chm_sp_carrier)
            self.kx0 = float(A["kx0"])
            self.carrier = torch.zeros(self.nx + 4, dtype=torch.complex64, device=dev)
        # fields
        D = S.Data
        fb = (self.nx, self.nkr, self.nm)
        sp = (self.nx, self.nr, self.nm)
        z = lambda shape: chimera.fortran_zeros(shape, torch.complex64, dev)  # noqa: E731
        self.EG = _c64(D["EG_fb"])
        self.Jfb = z(fb + (3,))
        self.Bfb = z(fb + (3,))
        self.EB = z(sp + (6,))
        if self.space_charge:
            self.Rfb = z(fb)
            self.gprv = _c64(D["gradRho_fb_prv"])
            self.gnxt = _c64(D["gradRho_fb_nxt"])
        n_grid = self.nx * self.nr * self.nm
        self.accJ = torch.zeros(n_grid * 3 * 2, dtype=torch.int64, device=dev)
        self.accR = torch.zeros(n_grid * 2, dtype=torch.int64, device=dev)
        self.accBG = torch.zeros(n_grid * 2, dtype=torch.int64, device=dev)
        self.ws = torch.empty(_lib.query("chm_sp_fb_ws_bytes", self.nx, self.nr, self.nkr, self.nm),
                              dtype=torch.uint8, device=dev)
        self.scale_ws = torch.empty(_lib.query("chm_sp_scale_ws_bytes"), dtype=torch.uint8,
                                    device=dev)
        # particles in deposit order (cell_order: serpentine patches of cells,
        # runs of 16 of the tile layout sharing a deposit cell)
        self.dr = float(A["dr"])
        self.parts = []
        self.order0 = []  # the initial permutation of each species (particle order of to_fp64)
        for spc in self.fp.Particles:
            P = _SpParticles(dev, spc.num_particles)
            d = spc.Data
            o = cell_order(d["coords"], self.X0, self.dx, self.dr)
            P.append_f64(d["coords"][:, o], d["momenta"][:, o], d["weights"][o], self.X0, self.dx)
            self.parts.append(P)
            self.order0.append(o)
        self.scaleJ = torch.zeros(2, dtype=torch.float64, device=dev)
        self.scaleR = torch.zeros(2, dtype=torch.float64, device=dev)
        self.scaleBG = torch.zeros(2, dtype=torch.float64, device=dev)
        self._scales_valid = False
        # absorbed particles are dropped from the arrays every this many
        # window moves (they are marked dead, with zero weight, meanwhile)
        self.compact_every = 32
        # the background density is deposited on window moves
        # (chimera_main.py:277-284); it starts empty, as the reference's
        self.have_bg = False
        self._bg_key = None  # still particles' layout at the last full background deposit
        self._bg_ext = None  # per-block cell ranges of that deposit (device int2)
        for spc, P in self._still():  # (allocated here, outside any graph capture)
            self._bg_ext = torch.empty(2 * ((P.cap + 2047) // 2048), dtype=torch.int32,
                                       device=dev)
        self.bg_shift = True  # move the background with whole-cell window moves
        self._inject_order = {}  # particle order of injected batches, per shape
        # the device error flags (a tensor-core CTA that gave up on a wait, a
        # deposit cell outside its block box) are read every this many steps
        # and by check_status(); either raises
        self.check_every = 64
        self._steps = 0
        # re-sort by deposit cell every this many steps (0: never), or "auto":
        # SortCadence picks the cadence from measured times.  A sort changes
        # the order of the FP32 run sums of the deposit, so a fixed cadence
        # keeps runs bitwise reproducible; "auto" makes the sort steps (and
        # so the last bits of the fields) depend on timing.
        self.sort_every = 64
        self.sorter = SortCadence()
        self._since_sort = 0

    # ------------------------------------------------------------------
    def _moving(self):
        return [(spc, P) for spc, P in zip(self.fp.Particles, self.parts)
                if "Still" not in spc.Args["Features"]]

    def _still(self):
        return [(spc, P) for spc, P in zip(self.fp.Particles, self.parts)
                if "Still" in spc.Args["Features"]]

    def _win(self):
        """Window origin in cells from X0, k + f: the host mirror of the
        device record (chm_sp_window), f rounded to FP32 as the kernels read it."""
        return self._wk, float(np.float32(self._wfd))

    def _win_set(self, leftX):
        _lib.call("chm_sp_window_set", self.win.data_ptr(), float(leftX), self.X0, float(self.dx),
                  _stream())
        self._wk, self._wfd = window_cells(leftX, self.X0, self.dx)

    def _win_restore(self, k, fd):
        """Device record and host mirror with the cell position (k, fd)."""
        import struct
        raw = struct.pack("<ddddif", float(self.solver.Args["leftX"]), self.X0, float(self.dx),
                          fd, k, float(np.float32(fd)))
        buf = torch.frombuffer(bytearray(raw.ljust(self.win.numel(), b"\0")), dtype=torch.uint8)
        self.win.copy_(buf.to(self.device))
        self._wk, self._wfd = int(k), float(fd)

    def _win_after(self, shift):
        """(k, fd) after a move by shift, as chm_sp_window_advance computes them."""
        return window_cells_after(self._wk, self._wfd, shift, self.dx)

    def _win_advance(self, shift):
        _lib.call("chm_sp_window_advance", self.win.data_ptr(), float(shift), _stream())
        self._wk, self._wfd = self._win_after(shift)

    def _refresh_scales(self):
        """Global deposit scales from sum |w| (recomputed when particles change)."""
        st = _stream()
        mov = self._moving()
        # one species deposits into each accumulator in the benchmark; with
        # several, the largest bound times the species count is used
        for targets, group in (((self.scaleJ, self.scaleR), mov), ((self.scaleBG,), self._still())):
            if not group:
                for t in targets:
                    t.fill_(1.0)
                continue
            vals = []
            for spc, P in group:
                tmp = torch.empty(2, dtype=torch.float64, device=self.device)
                _lib.call("chm_sp_weight_scale", tmp.data_ptr(), P.buf["w"].data_ptr(), P.n,
                          self.scale_ws.data_ptr(), self.scale_ws.numel(), st)
                vals.append(tmp)
            if len(vals) == 1:
                for t in targets:
                    t.copy_(vals[0])
            else:
                B = torch.stack([v[1] for v in vals]).sum()
                e = torch.clamp(61.0 - torch.ceil(torch.log2(B)), max=120.0)
                for t in targets:
                    t[0] = torch.pow(2.0, e)
                    t[1] = B
        self._scales_valid = True

    def _deposit(self, P, push, accJ, accR, scaleJ, scaleR):
        k, f = self._win()
        if self.env:
            # (the envelope solver: push + J_z with the carrier; no charge)
            _lib.call("chm_sp_push_deposit_env", *P.ptrs(), P.n, k, f, 1.0 / self.dx,
                      float(self.solver.Args["dr_inv"]), float(self.dt), float(self.dx), self.nx,
                      self.nr, self.nm,
                      accJ.data_ptr(), scaleJ.data_ptr(), self.carrier.data_ptr(),
                      self.carrier.numel(), float(self.kx0 * self.dx), _stream(),
                      self.win.data_ptr())
            return
        _lib.call("chm_sp_push_deposit", *P.ptrs(), P.n, k, f, 1.0 / self.dx,
                  float(self.solver.Args["dr_inv"]), float(self.dt), self.nx, self.nr, self.nm,
                  int(push), accJ.data_ptr() if accJ is not None else None,
                  scaleJ.data_ptr() if scaleJ is not None else None,
                  accR.data_ptr() if accR is not None else None,
                  scaleR.data_ptr() if scaleR is not None else None, _stream(), self.win.data_ptr())

    def _bg_shift(self, wind):
        """Whole cells by which the background density can move with the
        window at this move instead of a full deposit
        (chm_sp_deposit_background): one still species whose particles are
        unchanged since the last full deposit, no absorption or injection,
        and a move of exactly n >= 1 cells that leaves the window's FP32
        fraction as it was (the device window record advances the same
        way); 0 for a full deposit.  Call before the move."""
        still = self._still()
        if (len(still) != 1 or self.nm > 3 or not self.have_bg or "AbsorbLayer" in wind
                or "AddPlasma" in wind):
            return 0
        P = still[0][1]
        if self._bg_key != (P.n, P.cap, *P.ptrs()):
            return 0

        k1, fd1 = self._win_after(wind["shiftX"])
        n = k1 - self._wk
        return n if (1 <= n < self.nx and np.float32(fd1) == np.float32(self._wfd)) else 0

    def _bg_plan(self, istep):
        """The background mode of step istep's window moves (for the graph key)."""
        if not (self.space_charge and "BckGrndRho" in self.solver.Data):
            return 0
        fp = self.fp
        out = 0
        for wind in fp.MovingFrames:
            if istep < wind["TimeActive"][0] or istep > wind["TimeActive"][1]:
                continue
            if np.mod(istep - wind["TimeActive"][0], wind["Steps"]) != 0:
                continue
            out = self._bg_shift(wind)
        return out

    def _deposit_background(self, shift_cells=0):
        if not self._scales_valid:
            self._refresh_scales()
        still = self._still()
        if len(still) != 1 or self.nm > 3 or still[0][1].n >= 2 ** 31 - 4096:
            self.accBG.zero_()
            for spc, P in still:
                self._deposit(P, False, None, self.accBG, None, self.scaleBG)
            self._bg_key = None
        else:
            # the run kernels' background pass: a full deposit that records each
            # block's cell range, or (shift_cells > 0) the grid moved with the
            # window and only the entering columns deposited
            P = still[0][1]
            if not shift_cells:
                self.accBG.zero_()
            nb = (P.cap + 2047) // 2048
            if self._bg_ext is None or self._bg_ext.numel() < 2 * nb:
                self._bg_ext = torch.empty(2 * nb, dtype=torch.int32, device=self.device)
            k, f = self._win()
            _lib.call("chm_sp_deposit_background", *P.ptrs(), P.n, k, f,
                      float(self.solver.Args["dr_inv"]), self.nx, self.nr, self.nm,
                      self.accBG.data_ptr(), self.scaleBG.data_ptr(), self._bg_ext.data_ptr(),
                      self._bg_ext.numel() // 2, int(shift_cells), _stream(), self.win.data_ptr())
            self._bg_key = (P.n, P.cap, *P.ptrs())
        self.have_bg = bool(still)

    def _fb_in(self, out, acc, scale, acc2, scale2, ncomp):
        A = self.solver.Args
        _lib.call("chm_sp_fb_in_acc", out.data_ptr(), acc.data_ptr(), scale.data_ptr(),
                  acc2.data_ptr() if acc2 is not None else None,
                  scale2.data_ptr() if scale2 is not None else None, float(A["leftX"]),
                  self.kxb64.data_ptr(), C.addressof(self.ops["InCurr"]), self.depfact.data_ptr(),
                  self.nx, self.nr, self.nkr, self.nm, ncomp, self.ws.data_ptr(), self.ws.numel(),
                  _stream(), self.win.data_ptr())

    # ------------------------------------------------------------------
    def make_step(self, istep):
        """chimera_main.py:82-92 in the split precision."""
        self._maybe_sort(istep)
        self._step_body(istep)
        self._after_step()

    # ------------------------------------------------------------------
    # CUDA-graph replay of a step
    def graph_capturable(self) -> bool:
        """A step is captured when its host side is the same every step: a
        window without plasma injection or absorbing layer (those draw host
        random numbers or read counts back) and a fixed re-sort cadence."""
        for wind in self.fp.MovingFrames:
            if "AddPlasma" in wind or wind.get("AbsorbLayer", 0) > 0:
                return False
        return self.sort_every != "auto"

    def _layout_key(self, istep):
        # the particle arrays and counts; which charge-gradient buffer holds
        # the previous step's gradient (the step swaps the two) and whether
        # the step's background deposit is full or a shift
        gp = self.gprv.data_ptr() if self.space_charge else 0
        bg = self._bg_plan(istep) if self.bg_shift else 0
        return tuple((P.n, P.cap, *P.ptrs()) for P in self.parts) + ((gp, bg),)

    def graph_step(self, istep):
        """make_step(istep) with the step's kernels replayed from a CUDA graph.
        The graph holds the device work of one step (window origin advance,
        deposits, spectral stage, gather and push); it is captured on the
        second call (the first step runs eagerly, so that the tensor-core
        products can time their tile widths) and again whenever the particle
        arrays change (a re-sort, compaction or growth).  The host side (window bookkeeping, re-sorts,
        error-flag reads) runs outside the graph.  Same results as
        make_step, bitwise.  Falls back to make_step when the step is not
        capturable (see graph_capturable)."""
        if not self.graph_capturable():
            return self.make_step(istep)
        if not getattr(self, "_eager_done", False):
            # the first step runs eagerly: the tensor-core products time their
            # column-tile widths on a shape's first launch, which a capture cannot
            self._eager_done = True
            return self.make_step(istep)
        self._maybe_sort(istep)
        if not self._scales_valid:
            self._refresh_scales()
        key = self._layout_key(istep)
        graphs = getattr(self, "_graphs", None)
        if graphs is None or graphs[0] != key[:-1]:
            graphs = self._graphs = [key[:-1], {}]  # per gradient-buffer assignment
        self._graph = graphs[1].get(key[-1])
        if self._graph is None:
            lib = _lib.load()
            g = torch.cuda.CUDAGraph()
            n0 = lib.chm_launch_count()
            with torch.cuda.graph(g):
                self._step_body(istep)
            self.graph_launches = lib.chm_launch_count() - n0  # kernels per replay
            self._graph = graphs[1][key[-1]] = g
            self.graph_captures = getattr(self, "graph_captures", 0) + 1
        else:
            self._host_effects(istep)
        self._graph.replay()
        self.graph_replays = getattr(self, "graph_replays", 0) + 1
        self._after_step()

    def _host_effects(self, istep):
        """The host side of a replayed step: the window moves' Xgrid / leftX /
        rightX bookkeeping (chimera_main.py:286-304) and the swap of the two
        charge-gradient buffers."""
        if self.space_charge:
            self.gprv, self.gnxt = self.gnxt, self.gprv
        fp = self.fp
        for wind in fp.MovingFrames:
            if istep < wind["TimeActive"][0] or istep > wind["TimeActive"][1]:
                continue
            if np.mod(istep - wind["TimeActive"][0], wind["Steps"]) != 0:
                continue
            # (the device record advances inside the graph; the host mirror here)
            fp.move_frame(wind)
            self._wk, self._wfd = self._win_after(wind["shiftX"])
            if "Staged" in wind["Features"]:
                fp.move_frame(wind)
                self._wk, self._wfd = self._win_after(wind["shiftX"])

    def _after_step(self):
        self._steps += 1
        self._since_sort += 1
        if self.check_every and self._steps % self.check_every == 0:
            self.check_status()

    def _step_body(self, istep):
        fp = self.fp
        A = self.solver.Args
        st = _stream()
        ws, wsb = self.ws.data_ptr(), self.ws.numel()
        staged_move = False
        # window, stage 1 (chimera_main.py:292-302)
        for wind in fp.MovingFrames:
            if istep < wind["TimeActive"][0] or istep > wind["TimeActive"][1]:
                continue
            if np.mod(istep - wind["TimeActive"][0], wind["Steps"]) != 0:
                continue
            if "Staged" in wind["Features"]:
                staged_move = True
            if wind.get("AbsorbLayer", 0) > 0:
                prof = A.get("_damp32")
                if prof is None:
                    prof = A["_damp32"] = _f32(A["damp_profile"].cpu().numpy()
                                               if isinstance(A["damp_profile"], torch.Tensor)
                                               else A["damp_profile"], self.device)
                _lib.call("chm_sp_fb_filtr", self.EG.data_ptr(), float(A["leftX"]),
                          self.kx64.data_ptr(), prof.data_ptr(), prof.numel(), 0, self.nx,
                          self.nkr, self.nm, 6, ws, wsb, st, self.win.data_ptr())
            bg_shift = self._bg_shift(wind) if self.bg_shift else 0
            fp.move_frame(wind)
            self._win_advance(wind["shiftX"])
            if "AddPlasma" in wind:
                self._add_plasma(wind)
            if "AbsorbLayer" in wind:
                self._absorb(wind)
            if self.space_charge and "BckGrndRho" in self.solver.Data:
                self._deposit_background(bg_shift)
            # the reference's dep_dens here (postframe_corr) is overwritten by
            # project_density before any use; it is not repeated
        if not self._scales_valid:
            self._refresh_scales()
        ev = None
        if self.sort_every == "auto":
            ev = self.sorter.step_events(self._since_sort)
            ev[0].record()
        # push_coords + J (half step) [+ rho (new position), fused unless a
        # staged frame moves between the two deposits]
        self.accJ.zero_()
        fuse_rho = self.space_charge and not staged_move
        if self.space_charge:
            self.accR.zero_()
        if self.env:
            self._carrier()
        for spc, P in self._moving():
            self._deposit(P, True, self.accJ, self.accR if fuse_rho else None, self.scaleJ,
                          self.scaleR if fuse_rho else None)
        if "NoCurrent" in A["Features"]:
            self.Jfb.zero_()
        else:
            self._fb_in(self.Jfb, self.accJ, self.scaleJ, None, None, 3)
        # window, stage 2
        for wind in fp.MovingFrames:
            if istep < wind["TimeActive"][0] or istep > wind["TimeActive"][1]:
                continue
            if np.mod(istep - wind["TimeActive"][0], wind["Steps"]) != 0:
                continue
            if "Staged" in wind["Features"]:
                fp.move_frame(wind)
                self._win_advance(wind["shiftX"])
        # density
        if self.space_charge:
            if not fuse_rho:
                for spc, P in self._moving():
                    self._deposit(P, False, None, self.accR, None, self.scaleR)
            self.gprv, self.gnxt = self.gnxt, self.gprv
            bg = self.accBG if self.have_bg else None
            self._fb_in(self.Rfb, self.accR, self.scaleR, bg, self.scaleBG if bg is not None else None,
                        1)
            _lib.call("chm_sp_fb_grad", self.gnxt.data_ptr(), self.Rfb.data_ptr(),
                      C.addressof(self.ops["Dp"]), C.addressof(self.ops["Dm"]),
                      self.kx32.data_ptr(), self.nx, self.nkr, self.nm, ws, wsb, st)
        # fields: the Poisson correction (solvers.py:301-331) with the PSATD
        # update (solvers.py:281-299) fused into its last J update
        if self.poisson:
            _lib.call("chm_sp_poisson_psatd", self.Jfb.data_ptr(),
                      self.gprv.data_ptr() if self.space_charge else None,
                      self.gnxt.data_ptr() if self.space_charge else None, self.pf.data_ptr(),
                      float(A["dt_inv"]), C.addressof(self.ops["Dp"]), C.addressof(self.ops["Dm"]),
                      self.kx32.data_ptr(), self.nx, self.nkr, self.nm, 3, int(self.space_charge),
                      self.EG.data_ptr(), self.c1.data_ptr(), self.c2.data_ptr(), int(self.nterm),
                      ws, wsb, st)
        elif self.complex_psatd:
            # maxwell_push_wo_spchrg with the envelope solver's complex coefficients
            _lib.call("chm_sp_psatd_c", self.EG.data_ptr(), self.Jfb.data_ptr(), self.c1.data_ptr(),
                      self.c2.data_ptr(), self.nx * self.nkr * self.nm, st)
        else:
            P_ = self.nx * self.nkr * self.nm
            _lib.call("chm_sp_psatd", self.EG.data_ptr(), self.Jfb.data_ptr(),
                      self.gprv.data_ptr() if self.space_charge else None,
                      self.gnxt.data_ptr() if self.space_charge else None, self.c1.data_ptr(),
                      self.c2.data_ptr(), int(self.nterm), P_, st)
        self._project_fields_and_push()
        if ev is not None:
            ev[1].record()
        for spc, P in self._moving():
            _lib.call("chm_sp_count_live", P.counters.data_ptr(), P.n, st)

    def _maybe_sort(self, istep):
        every = self.sorter.cadence if self.sort_every == "auto" else int(self.sort_every or 0)
        if every and self._since_sort >= every:
            self.resort(istep)

    def resort(self, istep=None):
        """Re-sort every species by deposit cell (dead particles dropped)."""
        k, f = self._win()
        auto = self.sort_every == "auto"
        if auto:
            ev = self.sorter.sort_events()
            ev[0].record()
        for spc, P in zip(self.fp.Particles, self.parts):
            P.sort_cells(k, f, self.nx, self.nr, float(self.solver.Args["dr_inv"]))
        if auto:
            ev[1].record()
            ev[1].synchronize()
            self.sorter.update(self._steps if istep is None else istep)
        self._since_sort = 0

    def check_status(self):
        """Raise if a device error flag is set: a tensor-core product CTA
        that gave up on a bounded wait (its tile was not written) or deposit
        cells dropped outside their block box (corrupt positions).  Reading
        the flags waits for the work queued so far."""
        lib = _lib.load()
        umma = lib.chm_sp_umma_status()
        dropped = lib.chm_sp_deposit_dropped()
        if umma or dropped:
            raise _lib.ChimeraError(
                f"split form: tensor-core status {umma}, {dropped} deposit cells dropped")

    def _project_fields_and_push(self):
        A = self.solver.Args
        st = _stream()
        ws, wsb = self.ws.data_ptr(), self.ws.numel()
        if "NoPush" in A["Features"]:
            self.EB.zero_()
            return
        G = self.EG[:, :, :, 3:]
        env = "_env" if self.env else ""
        _lib.call("chm_sp_rot_b" + env, self.Bfb.data_ptr(), G.data_ptr(), self.pf.data_ptr(),
                  C.addressof(self.ops["Dp"]), C.addressof(self.ops["Dm"]), self.kx32.data_ptr(),
                  self.nx, self.nkr, self.nm, ws, wsb, st)
        _lib.call("chm_sp_fb_eb_out" + env, self.EB.data_ptr(), self.EG.data_ptr(),
                  self.Bfb.data_ptr(), float(A["leftX"]), self.kxb64.data_ptr(),
                  C.addressof(self.ops["Out"]), self.nx, self.nr, self.nkr, self.nm, ws, wsb, st,
                  self.win.data_ptr())
        k, f = self._win()
        if self.env:
            self._carrier()  # (a staged frame moved since the deposit)
        for i, (spc, P) in enumerate(zip(self.fp.Particles, self.parts)):
            if "Still" in spc.Args["Features"]:
                continue
            dtq = spc.Args["push_fact"] * spc.Args["TimeStep"]
            if not self.env:
                _lib.call("chm_sp_gather_push", *P.ptrs(), P.n, k, f, float(A["dr_inv"]),
                          self.EB.data_ptr(), self.nx, self.nr, self.nm, float(dtq), st,
                          self.win.data_ptr())
                continue
            und = self.undulators[i]
            prm = np.zeros(5)
            amap = None
            if und is not None:
                prm[:min(5, und[1].size)] = und[1][:5]
                amap = und[2]
            _lib.call("chm_sp_gather_push_env", *P.ptrs(), P.n, k, f, float(A["dr_inv"]),
                      self.EB.data_ptr(), self.nx, self.nr, self.nm, float(dtq),
                      self.carrier.data_ptr(), self.carrier.numel(), float(self.kx0 * self.dx),
                      0 if und is None else und[0], prm.ctypes.data,
                      None if amap is None else amap.data_ptr(),
                      0 if amap is None else amap.shape[0], self.X0, float(self.dx), st,
                      self.win.data_ptr())

    def _carrier(self):
        """The carrier table of the window's cells (chm_sp_carrier) from the
        device window record."""
        k, _ = self._win()
        _lib.call("chm_sp_carrier", self.carrier.data_ptr(), self.carrier.numel(), self.kx0,
                  self.X0, float(self.dx), k, _stream(), self.win.data_ptr())

    def _add_plasma(self, wind):
        fp = self.fp
        xsteps = int(wind["shiftX"] / wind["TimeStep"]) + 1
        idx = {id(s): i for i, s in enumerate(fp.Particles)}
        def ordered(spc, parts):
            # device-generated batches: the order from the host pattern
            # positions (the same for every batch of a shape, as cell_order
            # keys x relative to the batch's first cell), cached on the device
            xr = getattr(spc, "last_gen_xr", None)
            n = int(parts[0].shape[1])
            if xr is not None and xr[0].shape[0] == n:
                key = (id(spc), n, xsteps)
                o = self._inject_order.get(key)
                if o is None:
                    x, r = xr
                    o = torch.from_numpy(cell_order(np.vstack([x, r, 0.0 * r]), self.X0, self.dx,
                                                    self.dr)).to(self.device)
                    self._inject_order[key] = o
                spc.last_gen_xr = None
            else:
                o = cell_order(parts[0], self.X0, self.dx, self.dr)
            return [parts[0][:, o], parts[1][:, o], parts[2][o]]

        # the particles are built on the device (Specie.gen_parts_device: the
        # host draws the reference's random numbers, the kernel the rest)
        if "IonsOnTop" in wind["Features"]:
            s1, s2 = fp.Particles[:2]
            parts = ordered(s1, s1.gen_parts_device(Xsteps=xsteps, ProfileFunc=wind["AddPlasma"]))
            self.parts[idx[id(s1)]].append_f64(*parts, self.X0, self.dx)
            parts[-1] = parts[-1] * -1
            self.parts[idx[id(s2)]].append_f64(*parts, self.X0, self.dx)
        else:
            for s in fp.Particles:
                parts = ordered(s, s.gen_parts_device(Xsteps=xsteps, ProfileFunc=wind["AddPlasma"]))
                self.parts[idx[id(s)]].append_f64(*parts, self.X0, self.dx)
        self._scales_valid = False

    def _absorb(self, wind):
        """species.py:351-398 absorption (SimDom test) on the split layout:
        marks in place (compacting every ``compact_every`` window moves) and
        refreshes the deposit scales in the same pass."""
        scales = {}
        for spc, P in zip(self.fp.Particles, self.parts):
            if P.n == 0:
                continue
            a = spc.Args
            k, f = self._win()
            # species grid box in window cells
            xmin = (a["leftX"] + wind["AbsorbLayer"] * a["dx"] - self.solver.Args["leftX"]) / self.dx
            xmax = (a["rightX"] - self.solver.Args["leftX"]) / self.dx
            b = P.buf
            sc = torch.empty(2, dtype=torch.float64, device=self.device)
            _lib.call("chm_sp_absorb", b["ix"].data_ptr(), b["fx"].data_ptr(), b["y"].data_ptr(),
                      b["z"].data_ptr(), b["w"].data_ptr(), P.dead.data_ptr(), P.n, k, f,
                      float(xmin), float(xmax), float(a["upperR"] ** 2),
                      P.counters.data_ptr(), sc.data_ptr(), self.scale_ws.data_ptr(),
                      self.scale_ws.numel(), _stream())
            scales[id(P)] = sc
            P.moves += 1
            if P.moves >= self.compact_every:
                P.compact()
        # with one species per accumulator the absorbing pass gives the scales
        mov, still = self._moving(), self._still()
        if (len(mov) == 1 and len(still) <= 1 and id(mov[0][1]) in scales
                and (not still or id(still[0][1]) in scales)):
            self.scaleJ.copy_(scales[id(mov[0][1])])
            self.scaleR.copy_(scales[id(mov[0][1])])
            if still:
                self.scaleBG.copy_(scales[id(still[0][1])])
            self._scales_valid = True
        else:
            self._scales_valid = False

    # ------------------------------------------------------------------
    @property
    def num_moving(self) -> int:
        """Particles held by the moving species, dead ones not yet compacted
        included (an upper bound of the live count)."""
        return sum(P.n for _, P in self._moving())

    def live_particle_steps(self) -> int:
        """Sum over the steps made of the live moving particles after each
        step (one device->host read)."""
        return int(sum(int(P.counters[1].item()) for _, P in self._moving()))

    # ------------------------------------------------------------------
    # checkpoints: the FP64 run's drop_snap keys plus the split form's own
    # state (deposit scales, background accumulator) under ``split/``
    def drop_snap(self, fname="./snap_", verbose=False):
        """chimera_main.py:325-369 for the split form: ``to_fp64()`` (which
        compacts the particle arrays, in their split order) and the FP64
        keys, plus ``split/...``; returns the file name."""
        from . import snapshot
        self.to_fp64()
        arrays = snapshot.snap_arrays(self.fp.Solvers, self.fp.Particles, verbose)
        arrays["split/scaleJ"] = self.scaleJ.cpu().numpy()
        arrays["split/scaleR"] = self.scaleR.cpu().numpy()
        arrays["split/scaleBG"] = self.scaleBG.cpu().numpy()
        arrays["split/scales_valid"] = np.asarray(self._scales_valid)
        arrays["split/have_bg"] = np.asarray(self.have_bg)
        arrays["split/since_sort"] = np.asarray(self._since_sort)
        arrays["split/accBG"] = self.accBG.cpu().numpy()
        arrays["split/win"] = np.array([self._wk, self._wfd], dtype=np.float64)
        return snapshot.write(snapshot.snap_name(fname), arrays)

    def read_snap(self, fname="./test.npz", verbose=False):
        """chimera_main.py:371-410 for the split form: the FP64 Data / Args,
        then the split fields and particles from them (particles in the
        stored order), and the split state; a restart continues bitwise as
        the run that wrote the file."""
        from . import snapshot
        with np.load(fname, allow_pickle=False) as f:
            snapshot.read_into(f, self.fp.Solvers, self.fp.Particles, verbose)
            D = self.solver.Data
            self._win_set(float(self.solver.Args["leftX"]))
            if "split/win" in f.files:
                # the window's cell position as the writing run carried it
                k, fd = f["split/win"]
                self._win_restore(int(k), float(fd))
            self.EG.copy_(D["EG_fb"])
            if self.space_charge:
                self.gprv.copy_(D["gradRho_fb_prv"])
                self.gnxt.copy_(D["gradRho_fb_nxt"])
            for spc, P in zip(self.fp.Particles, self.parts):
                P.n = 0
                P.moves = 0
                P.counters.zero_()
                d = spc.Data
                P.append_f64(d["coords"], d["momenta"], d["weights"], self.X0, self.dx)
            # (the background's block ranges belong to the particles before the
            # read: the next window move deposits the background in full)
            self._bg_key = None
            if "split/scaleJ" in f.files:
                for t, k in ((self.scaleJ, "scaleJ"), (self.scaleR, "scaleR"),
                             (self.scaleBG, "scaleBG"), (self.accBG, "accBG")):
                    t.copy_(torch.from_numpy(np.ascontiguousarray(f["split/" + k])))
                self._scales_valid = bool(f["split/scales_valid"])
                self.have_bg = bool(f["split/have_bg"])
                if "split/since_sort" in f.files:
                    self._since_sort = int(f["split/since_sort"])
            else:
                self._scales_valid = False
                self.have_bg = False
                if self.space_charge and "BckGrndRho" in D and self._still():
                    self._deposit_background()
        return self

    def to_fp64(self):
        """Write the split state into the FP64 Data of the solver and species."""
        self.check_status()
        D = self.solver.Data
        D["EG_fb"].copy_(self.EG)
        D["EB"].copy_(self.EB)
        D["J_fb"].copy_(self.Jfb)
        D["B_fb"].copy_(self.Bfb)
        if self.space_charge:
            D["Rho_fb"].copy_(self.Rfb)
            D["gradRho_fb_nxt"].copy_(self.gnxt)
            D["gradRho_fb_prv"].copy_(self.gprv)
        for spc, P in zip(self.fp.Particles, self.parts):
            P.compact()
            spc.store.resize(P.n)
            spc._sync()
            d = spc.Data
            _lib.call("chm_sp_to_f64", *P.ptrs(), P.n, d["coords"].data_ptr(), d["coords"].stride(0),
                      d["coords"].stride(1), d["momenta"].data_ptr(), d["momenta"].stride(0),
                      d["momenta"].stride(1), d["weights"].data_ptr(), d["weights"].stride(0),
                      self.X0, self.dx, _stream())
        return self


def transform_errors(run: SplitRun) -> dict:
    """Relative L2 error of each split transform against the FP64 kernels on
    the run's own current data (converted exactly to FP64): fb_in of the last
    current deposit (the int64 accumulators, with DepFact), fb_grad of the
    charge spectrum, the 3-iteration Poisson correction of J_fb, curl +
    PoissFact of G and fb_eb_out with eb_correction of E and B.  Leaves the
    run's state unchanged."""
    S, A = run.solver, run.solver.Args
    nx, nr, nkr, nm = run.nx, run.nr, run.nkr, run.nm
    st = _stream()
    ws, wsb = run.ws.data_ptr(), run.ws.numel()
    dev = run.device
    c128 = lambda t: t.to(torch.complex128)  # noqa: E731
    rel = lambda a, b: float(torch.linalg.vector_norm(a.to(torch.complex128) - b)  # noqa: E731
                             / torch.linalg.vector_norm(b))
    errs = {}
    leftX = float(A["leftX"])
    # fb_in of the current accumulators
    acc = run.accJ.view(3, nm, nr, nx, 2).permute(3, 2, 1, 0, 4)  # (nx, nr, nm, 3, {re, im})
    J = torch.complex(acc[..., 0].to(torch.float64), acc[..., 1].to(torch.float64))
    J = J / run.scaleJ[0]
    J[:, 1] -= J[:, 0]
    J[:, 0] = 0
    Jf = chimera.fortran_empty(tuple(J.shape), torch.complex128, dev)
    Jf.copy_(J)
    del J
    out = chimera.fortran_zeros((nx, nkr, nm, 3), torch.complex64, dev)
    _lib.call("chm_sp_fb_in_acc", out.data_ptr(), run.accJ.data_ptr(), run.scaleJ.data_ptr(), None,
              None, leftX, run.kxb64.data_ptr(), C.addressof(run.ops["InCurr"]),
              run.depfact.data_ptr(), nx, nr, nkr, nm, 3, ws, wsb, st, None)
    ref = chimera._fb_in(chimera.fortran_zeros((nx, nkr, nm, 3), device=dev), Jf, leftX,
                         *A["FBCurrIn"], 3, fact=S.dev["DepFact"])
    errs["fb_in"] = rel(out, ref)
    del Jf, ref
    FBD = (A["DpS2S"], A["DmS2S"], A["kx"])
    if run.space_charge:
        g = chimera.fortran_zeros((nx, nkr, nm, 3), torch.complex64, dev)
        _lib.call("chm_sp_fb_grad", g.data_ptr(), run.Rfb.data_ptr(), C.addressof(run.ops["Dp"]),
                  C.addressof(run.ops["Dm"]), run.kx32.data_ptr(), nx, nkr, nm, ws, wsb, st)
        ref = chimera.fb_grad(chimera.fortran_zeros((nx, nkr, nm, 3), device=dev), c128(run.Rfb),
                              *FBD)
        errs["fb_grad"] = rel(g, ref)
        del g, ref
    if run.poisson:
        Js = run.Jfb.clone(memory_format=torch.preserve_format)
        sc = run.space_charge
        _lib.call("chm_sp_poisson", Js.data_ptr(), run.gprv.data_ptr() if sc else None,
                  run.gnxt.data_ptr() if sc else None, run.pf.data_ptr(), float(A["dt_inv"]),
                  C.addressof(run.ops["Dp"]), C.addressof(run.ops["Dm"]), run.kx32.data_ptr(),
                  nx, nkr, nm, 3, int(sc), ws, wsb, st)
        Jd = c128(run.Jfb)
        for _ in range(3):
            v = Jd.clone(memory_format=torch.preserve_format)
            v = chimera.fb_graddiv(v, *FBD)
            if sc:
                Jd = chimera.poiss_corr(Jd, v, c128(run.gprv), c128(run.gnxt), A["dt_inv"],
                                        S.dev["PoissFact"])
            else:
                Jd = chimera.omp_add_vec(Jd, chimera.omp_mult_vec(v, S.dev["PoissFact"]))
        errs["poisson"] = rel(Js, Jd)
        del Js, Jd, v
    G = run.EG[:, :, :, 3:]
    env = "_env" if run.env else ""
    Bs = chimera.fortran_zeros((nx, nkr, nm, 3), torch.complex64, dev)
    _lib.call("chm_sp_rot_b" + env, Bs.data_ptr(), G.data_ptr(), run.pf.data_ptr(),
              C.addressof(run.ops["Dp"]), C.addressof(run.ops["Dm"]), run.kx32.data_ptr(), nx, nkr,
              nm, ws, wsb, st)
    Gd = chimera.fortran_empty((nx, nkr, nm, 3), torch.complex128, dev)
    Gd.copy_(G)
    rot = chimera.fb_rot_env if run.env else chimera.fb_rot
    ref = rot(chimera.fortran_zeros((nx, nkr, nm, 3), device=dev), Gd, *FBD)
    ref = chimera.omp_mult_vec(ref, S.dev["PoissFact"])
    errs["rot_b"] = rel(Bs, ref)
    del Gd, ref
    EB = chimera.fortran_zeros((nx, nr, nm, 6), torch.complex64, dev)
    _lib.call("chm_sp_fb_eb_out" + env, EB.data_ptr(), run.EG.data_ptr(), Bs.data_ptr(), leftX,
              run.kxb64.data_ptr(), C.addressof(run.ops["Out"]), nx, nr, nkr, nm, ws, wsb, st, None)
    ref = chimera.fb_eb_out(chimera.fortran_zeros((nx, nr, nm, 6), device=dev), c128(run.EG),
                            c128(Bs), leftX, *A["FBout"], eb_mode=2 if run.env else 1)
    errs["fb_eb_out"] = rel(EB, ref)
    del EB, ref, Bs
    run.check_status()
    return errs
