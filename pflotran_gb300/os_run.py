"""Time-stepped operator-split run: a transport stand-in around the GPU
reaction step, one CUDA graph per step.

PFLOTRAN's operator-split mode alternates an explicit transport update of the
aqueous totals (`RTExplicitAdvection` with `TFluxTVD` and
`TVD_LIMITER_UPWIND`, src/pflotran/reactive_transport.F90:4501-4863,
transport.F90:958-1043) with `RTReact` over every cell
(reactive_transport.F90:1605-1806).  This driver does the same on a
structured grid of unit cells, entirely on one GPU:

* a log-normal permeability field exp(sigma_lnK * g), g a unit-variance
  Gaussian field with exponential covariance exp(-r / corr_len), synthesised
  by a seeded FFT spectral method;
* the steady Darcy pressure with a fixed head drop along x and no flow
  through the other faces (Jacobi-preconditioned conjugate gradients on the
  7-point two-point-flux operator with harmonic-mean transmissibilities),
  giving face fluxes;
* explicit first-order upwind advection of the totals with CFL sub-steps
  and a fixed inflow composition at x = 0, which drives a front through the
  domain;
* the reaction step (`ReactionStep.react_async`, learned warm start
  optional) over every cell.

Transport (one CUDA kernel per sub-step from libpfchem_transport.so on
precomputed per-cell upwind weights, or the flux form as torch tensor ops
with transport="torch"), a gather of the
sampled cells' pre-step state for the drift check and the reaction step are
captured into ONE CUDA graph, replayed once per step.  Transport is not part
of the chemistry library: the library's boundary is the reaction step, as
RTReact's is.
"""
from __future__ import annotations

import math
import time

import numpy as np

_STATE_FIELDS = ("total", "pri_molal", "ionic_strength", "mnrl_volfrac", "mnrl_area", "total_sorb_eq",
                 "eqionx_ref_cation_sorbed_conc", "srfcplxrxn_free_site_conc")
_OUT_FIELDS = ("pri_molal", "total_out", "mnrl_rate", "mnrl_volfrac", "total_sorb_eq", "ionic_strength",
               "sec_molal", "iterations", "status")


def lognormal_permeability(shape, sigma, corr_len, seed, device):
    """exp(sigma * g), g a zero-mean unit-variance Gaussian field whose
    covariance is exp(-r / corr_len) (periodic spectral synthesis; r in cells)."""
    import torch
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    freq = [torch.fft.fftfreq(s, device=device, dtype=torch.float64) * (2 * math.pi) for s in shape]
    k2 = freq[0][:, None, None] ** 2 + freq[1][None, :, None] ** 2 + freq[2][None, None, :] ** 2
    # the 3-D spectral density of exp(-r/l) is proportional to (1 + k^2 l^2)^-2
    amp = (1.0 + k2 * corr_len ** 2) ** -1.0
    noise = torch.randn(shape, generator=gen, device=device, dtype=torch.float64)
    g = torch.fft.ifftn(torch.fft.fftn(noise) * amp).real
    g = (g - g.mean()) / g.std()
    return torch.exp(sigma * g)


def _transmissibilities(K):
    hm = lambda a, b: 2.0 * a * b / (a + b)
    return hm(K[1:], K[:-1]), hm(K[:, 1:], K[:, :-1]), hm(K[:, :, 1:], K[:, :, :-1]), 2.0 * K[0], 2.0 * K[-1]


def darcy_fluxes(K, head_drop=1.0, rtol=1e-10, max_iter=20000):
    """Face fluxes (qx [nx+1,ny,nz], qy [nx,ny+1,nz], qz [nx,ny,nz+1]) of steady
    Darcy flow on unit cells: head `head_drop` at the west face, 0 at the
    east face, no flow through the others.  Returns (qx, qy, qz, iterations)."""
    import torch
    Tx, Ty, Tz, Tw, Te = _transmissibilities(K)
    diag = torch.zeros_like(K)
    diag[1:] += Tx
    diag[:-1] += Tx
    diag[:, 1:] += Ty
    diag[:, :-1] += Ty
    diag[:, :, 1:] += Tz
    diag[:, :, :-1] += Tz
    diag[0] += Tw
    diag[-1] += Te

    def A(p):
        r = diag * p
        r[1:] -= Tx * p[:-1]
        r[:-1] -= Tx * p[1:]
        r[:, 1:] -= Ty * p[:, :-1]
        r[:, :-1] -= Ty * p[:, 1:]
        r[:, :, 1:] -= Tz * p[:, :, :-1]
        r[:, :, :-1] -= Tz * p[:, :, 1:]
        return r

    b = torch.zeros_like(K)
    b[0] = Tw * head_drop
    # start from the homogeneous solution (linear head)
    nx = K.shape[0]
    p = head_drop * (1.0 - (torch.arange(nx, dtype=K.dtype, device=K.device) + 0.5) / nx)[:, None, None].expand_as(K)
    p = p.contiguous()
    r = b - A(p)
    z = r / diag
    d = z.clone()
    rz = (r * z).sum()
    bn = float(b.norm())
    it = 0
    for it in range(1, max_iter + 1):
        Ad = A(d)
        alpha = rz / (d * Ad).sum()
        p += alpha * d
        r -= alpha * Ad
        if it % 25 == 0 and float(r.norm()) < rtol * bn:
            break
        z = r / diag
        rz_new = (r * z).sum()
        d = z + (rz_new / rz) * d
        rz = rz_new
    nxx, ny, nz = K.shape
    qx = torch.zeros((nxx + 1, ny, nz), dtype=K.dtype, device=K.device)
    qx[1:-1] = Tx * (p[:-1] - p[1:])
    qx[0] = Tw * (head_drop - p[0])
    qx[-1] = Te * p[-1]
    qy = torch.zeros((nxx, ny + 1, nz), dtype=K.dtype, device=K.device)
    qy[:, 1:-1] = Ty * (p[:, :-1] - p[:, 1:])
    qz = torch.zeros((nxx, ny, nz + 1), dtype=K.dtype, device=K.device)
    qz[:, :, 1:-1] = Tz * (p[:, :, :-1] - p[:, :, 1:])
    return qx, qy, qz, it


def outflow_rate(qx, qy, qz):
    """Sum of outgoing face fluxes per cell."""
    pos = lambda q: q.clamp(min=0.0)
    neg = lambda q: (-q).clamp(min=0.0)
    return (pos(qx[1:]) + neg(qx[:-1]) + pos(qy[:, 1:]) + neg(qy[:, :-1]) + pos(qz[:, :, 1:]) + neg(qz[:, :, :-1]))


def upwind_advect(T, qx, qy, qz, pore_vol, dt_sub, inflow):
    """One explicit first-order upwind step of totals T [ncomp, nx, ny, nz]
    (mol/L of pore water); `inflow` [ncomp] enters through the west face,
    water leaves through the east face at its cell's composition."""
    import torch
    div = torch.zeros_like(T)  # net inflow of each component per cell
    qxi = qx[1:-1]
    f = qxi * torch.where(qxi > 0, T[:, :-1], T[:, 1:])
    div[:, 1:] += f
    div[:, :-1] -= f
    qw = qx[0]
    div[:, 0] += torch.where(qw > 0, qw * inflow[:, None, None], qw * T[:, 0])
    qe = qx[-1]
    div[:, -1] -= torch.where(qe > 0, qe * T[:, -1], torch.zeros_like(qe))
    qyi = qy[:, 1:-1]
    f = qyi * torch.where(qyi > 0, T[:, :, :-1], T[:, :, 1:])
    div[:, :, 1:] += f
    div[:, :, :-1] -= f
    qzi = qz[:, :, 1:-1]
    f = qzi * torch.where(qzi > 0, T[:, :, :, :-1], T[:, :, :, 1:])
    div[:, :, :, 1:] += f
    div[:, :, :, :-1] -= f
    return T + (dt_sub / pore_vol) * div


_transport_lib = None


def _transport():
    """libpfchem_transport.so (built with the chemistry library)."""
    global _transport_lib
    if _transport_lib is None:
        import ctypes as C
        import os
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libpfchem_transport.so")
        if not os.path.exists(path):
            from .build import build
            build()
        lib = C.CDLL(path)
        vp = C.c_void_p
        lib.pfchem_transport_upwind.argtypes = [vp] * 5 + [C.c_int] * 5 + [vp]
        lib.pfchem_transport_upwind.restype = C.c_int
        _transport_lib = lib
    return _transport_lib


def upwind_coefficients(qx, qy, qz, pore_vol, dt_sub):
    """Per-cell weights [7, nx, ny, nz] of one `upwind_advect` sub-step
    written as T' = a0 T + sum_f a_f T_f over the six neighbours f = west,
    east, south, north, bottom, top: a0 = 1 - s * (outgoing flux), a_f =
    s * (incoming flux through f) (0 where f is an outlet or closed), s =
    dt_sub / pore_vol.  The west weight of an x = 0 cell multiplies the
    inflow composition."""
    import torch
    s = dt_sub / pore_vol
    pos = lambda q: q.clamp(min=0.0)
    a = torch.stack([1.0 - s * outflow_rate(qx, qy, qz),
                     s * pos(qx[:-1]), s * pos(-qx[1:]),
                     s * pos(qy[:, :-1]), s * pos(-qy[:, 1:]),
                     s * pos(qz[:, :, :-1]), s * pos(-qz[:, :, 1:])])
    a[2, -1] = 0.0       # nothing enters through the east outlet
    a[3, :, 0] = 0.0     # closed y and z boundaries
    a[4, :, -1] = 0.0
    a[5, :, :, 0] = 0.0
    a[6, :, :, -1] = 0.0
    return a.contiguous()


def upwind_advect_cuda(T0, T1, tmp, coef, inflow, nsub, stream):
    """`nsub` sub-steps of `upwind_advect` (weights from
    `upwind_coefficients`) in one CUDA kernel each, from T0 into T1 (tmp:
    scratch like T1), enqueued on `stream`.  The same update as
    `upwind_advect` up to rounding (the weights are summed in another
    order)."""
    for t in (T0, T1, tmp, coef, inflow):
        if not (t.is_cuda and t.is_contiguous() and t.dtype == T0.dtype):
            raise ValueError("upwind_advect_cuda: contiguous float64 CUDA tensors expected")
    ncomp, nx, ny, nz = T0.shape
    if tuple(coef.shape) != (7, nx, ny, nz) or tuple(inflow.shape) != (ncomp,):
        raise ValueError("upwind_advect_cuda: coef [7, nx, ny, nz] and inflow [ncomp] expected")
    err = _transport().pfchem_transport_upwind(T0.data_ptr(), T1.data_ptr(), tmp.data_ptr(), coef.data_ptr(),
                                               inflow.data_ptr(), ncomp, nx, ny, nz, nsub, stream.cuda_stream)
    if err != 0:
        raise RuntimeError(f"pfchem_transport_upwind: CUDA error {err}")


def drift(net, gpu, ref, mask):
    """Max scaled relative differences GPU vs oracle over the `mask` cells:
    free-ion molalities (relative), aqueous totals (scaled by the sum of the
    terms of each total), mineral volume fractions (relative) and rates
    (scaled by rate constant x area)."""
    from .workloads import Speciator
    n = ref.ncells
    N = net.N
    out = {}
    if not mask.any():
        return out
    rel = lambda x, y, s: np.abs(x - y) / np.maximum(np.abs(y), s)
    out["pri_molal"] = float(rel(gpu.pri_molal.reshape(N, n), ref.pri_molal.reshape(N, n), 1e-300)[:, mask].max())
    m = ref.pri_molal.reshape(N, n)
    S = m.copy()
    if net.Nc:
        S = m + np.abs(Speciator(net).nu_np).T @ ref.sec_molal.reshape(-1, n)[:net.Nc]
    S = S * (ref.den_kg * 1e-3)[None, :]
    out["total"] = float(rel(gpu.total_out.reshape(N, n), ref.total_out.reshape(N, n), S)[:, mask].max())
    if net.Nm:
        k = np.array([mn.extra["k"] for mn in net.minerals])[:, None]
        area = ref.mnrl_area.reshape(-1, n)[:net.Nm]
        out["mnrl_rate"] = float(rel(gpu.mnrl_rate.reshape(-1, n)[:net.Nm], ref.mnrl_rate.reshape(-1, n)[:net.Nm],
                                     k * area)[:, mask].max())
        out["mnrl_volfrac"] = float(rel(gpu.mnrl_volfrac.reshape(-1, n)[:net.Nm],
                                        ref.mnrl_volfrac.reshape(-1, n)[:net.Nm], 1e-300)[:, mask].max())
    return out


class OperatorSplitRun:
    """State and captured step graph of the time-stepped problem."""

    def __init__(self, shape=(128, 128, 128), dt=86400.0, sigma=1.5, corr_len=10.0, seed=11, warm_start=True,
                 train_samples=2_097_152, epochs=8, autotune=True, drift_sample=512,
                 cells_per_step=2.0, courant=0.9, device="cuda", log=print, jacobian=0, transport="cuda",
                 mlp_backend=None):
        import torch
        from . import workloads
        from .lib import ReactionStep
        from .surrogate import fit, generate

        self.log = log or (lambda *a: None)
        self.shape = tuple(shape)
        self.n = n = int(np.prod(shape))
        self.dt = dt
        self.seed = seed
        self.drift_sample = min(int(drift_sample), n)
        self.device = device
        if transport not in ("cuda", "torch"):
            raise ValueError(f"transport: 'cuda' or 'torch', not {transport!r}")
        self.transport = transport
        net = workloads.synthetic_network()
        self.net = net
        _, self.opt, cells, _ = workloads.synthetic_cells(n, seed=seed, net=net, device=device)
        self.opt.jacobian = jacobian  # PFCHEM_JACOBIAN_*
        cells.sec_molal = np.zeros(max(net.Nc, 1) * n)
        d = cells.to_device(device)
        d.total_out.copy_(d.total)  # transport reads the previous step's aqueous totals
        self.cells = d
        self.step = ReactionStep(net, self.opt)
        if mlp_backend is not None:  # PFCHEM_MLP_*: tensor-core path of the warm start (library default: tcgen05)
            self.step.surrogate_backend(mlp_backend)
        self.report = {"train": None}
        if warm_start:
            t0 = time.perf_counter()
            X, molal = generate(self.step, lambda m, s: workloads.synthetic_cells(m, seed=s, net=net,
                                                                                  device=device)[2],
                                train_samples, seed + 101, dt)
            rep, _ = fit(self.step, X, molal, epochs=epochs)
            del X, molal
            self.step.surrogate_enable(True)
            self.report["train"] = {"samples": int(rep.samples), "final_loss": float(rep.final_loss),
                                    "s": time.perf_counter() - t0}
        if autotune:
            trial = d.copy()
            self.step.autotune(trial, dt)
            del trial
        L = self.step.launch()
        self.report["launch"] = {"block_threads": L.block_threads, "blocks_per_sm": L.blocks_per_sm,
                                 "refill_min_idle": L.refill_min_idle}
        self.step.reserve(n)
        # flow field
        t0 = time.perf_counter()
        K = lognormal_permeability(self.shape, sigma, corr_len, seed, device)
        qx, qy, qz, cg_its = darcy_fluxes(K)
        por = float(cells.porosity[0])
        self.pore_vol = por  # unit cells: pore volume per cell in m^3
        # scale the fluxes so that the mean pore velocity along x is
        # `cells_per_step` cells per reaction step
        v = float(qx[1:-1].mean()) / self.pore_vol
        scale = cells_per_step / (v * dt)
        self.qx, self.qy, self.qz = qx * scale, qy * scale, qz * scale
        out_max = float(outflow_rate(self.qx, self.qy, self.qz).max())
        self.nsub = max(1, int(math.ceil(dt * out_max / self.pore_vol / courant)))
        torch.cuda.synchronize()
        self.report["flow"] = {"cg_iterations": cg_its, "s": time.perf_counter() - t0, "substeps": self.nsub,
                               "transport": transport,
                               "lnK_std": float(torch.log(K).std()), "max_cell_courant": dt * out_max / self.pore_vol}
        # inflow water: the equilibrium totals of one cell of the same distribution
        _, _, w, _ = workloads.synthetic_cells(1, seed=seed + 7, net=net, device=device)
        self.inflow = torch.as_tensor(w.total, device=device)
        self.tmp = self.coef = None
        if transport == "cuda":
            self.tmp = torch.empty_like(d.total)
            self.coef = upwind_coefficients(self.qx, self.qy, self.qz, self.pore_vol, dt / self.nsub)
        # sampled cells for the drift check (indices refreshed before each replay)
        self.idx = torch.zeros(self.drift_sample, dtype=torch.long, device=device)
        self.snap = {f: torch.empty((getattr(d, f).numel() // n, self.drift_sample), dtype=torch.float64,
                                    device=device)
                     for f in _STATE_FIELDS if getattr(d, f) is not None}
        self.graph = None

    def _step_body(self, stream, ev=None):
        import torch
        d = self.cells
        N = self.net.N
        if self.transport == "cuda":
            shp = (N,) + self.shape
            upwind_advect_cuda(d.total_out.view(shp), d.total.view(shp), self.tmp.view(shp), self.coef, self.inflow,
                               self.nsub, stream)
        else:
            T = d.total_out.view(N, *self.shape)
            for _ in range(self.nsub):
                T = upwind_advect(T, self.qx, self.qy, self.qz, self.pore_vol, self.dt / self.nsub, self.inflow)
            d.total.copy_(T.reshape(-1))
        for f, buf in self.snap.items():
            a = getattr(d, f)
            torch.index_select(a.view(-1, self.n), 1, self.idx, out=buf)
        if ev is not None:
            ev[0].record(stream)
        self.step.react_async(d, self.dt, stream)
        if ev is not None:
            ev[1].record(stream)

    def capture(self):
        """Captures transport + sample gather + reaction step into one graph."""
        import torch
        self.ev = None
        try:
            self.ev = [torch.cuda.Event(enable_timing=True, external=True) for _ in range(2)]
        except TypeError:
            self.ev = None
        try:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, capture_error_mode="thread_local"):
                self._step_body(torch.cuda.current_stream(), self.ev)
        except RuntimeError:
            if self.ev is None:
                raise
            # timing events inside a graph need external event records; do without
            self.ev = None
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, capture_error_mode="thread_local"):
                self._step_body(torch.cuda.current_stream(), None)
        self.graph = g

    def run(self, steps=50, oracle_fn=None):
        """Replays the step graph `steps` times; returns per-step records."""
        import torch
        if self.graph is None:
            self.capture()
        net, N, n = self.net, self.net.N, self.n
        rng = np.random.default_rng(self.seed + 12345)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        records = []
        for s in range(steps):
            idx = np.sort(rng.choice(n, self.drift_sample, replace=False))
            self.idx.copy_(torch.as_tensor(idx, device=self.device))
            torch.cuda.synchronize()
            e0.record()
            self.graph.replay()
            e1.record()
            torch.cuda.synchronize()
            step_ms = e0.elapsed_time(e1)
            st = self.step.async_stats()
            rec = {"step": s + 1, "step_ms": step_ms, "nonconverged": int(st.nonconverged),
                   "mean_iterations": st.sum_iterations / n, "max_iterations": int(st.max_iterations),
                   "warm_start_used": int(st.alt_guess_used)}
            if self.ev is not None:
                rec["react_ms"] = self.ev[0].elapsed_time(self.ev[1])
                rec["transport_ms"] = step_ms - rec["react_ms"]
                rec["solves_per_s"] = n / (rec["react_ms"] * 1e-3)
            rec["step_solves_per_s"] = n / (step_ms * 1e-3)
            it = self.cells.iterations
            rec["iteration_histogram"] = torch.bincount(it.long().clamp(min=0), minlength=1).cpu().tolist()
            if oracle_fn is not None and self.drift_sample:
                rec["drift"] = self._drift(idx, oracle_fn)
            records.append(rec)
            self.log(f"step {s + 1}: {rec.get('solves_per_s', rec['step_solves_per_s']) / 1e6:.2f} M solves/s, "
                     f"mean its {rec['mean_iterations']:.2f}, max {rec['max_iterations']}, "
                     f"drift {rec.get('drift')}")
        return records

    def run_eager(self, steps=1):
        """The same steps without the graph (launch by launch), for checking
        that the captured step computes the same thing."""
        import torch
        for _ in range(steps):
            self._step_body(torch.cuda.current_stream(), None)
            torch.cuda.synchronize()

    def _drift(self, idx, oracle_fn):
        """Runs the oracle RReact on the sampled cells' pre-step state and
        compares it with the GPU's post-step state."""
        import torch
        from .cells import CellBatch
        net, N, n = self.net, self.net.N, self.n
        m = len(idx)
        d = self.cells
        ref = CellBatch(m)
        for f in ("temperature", "saturation", "den_kg", "porosity", "volume", "soil_particle_density"):
            a = getattr(d, f)
            if a is not None:
                setattr(ref, f, a[torch.as_tensor(idx, device=a.device)].cpu().numpy())
        for f, buf in self.snap.items():
            setattr(ref, f, buf.cpu().numpy().ravel().copy())
        ref.total_out = np.zeros(N * m)
        ref.mnrl_rate = np.zeros(max(net.Nm, 1) * m)
        ref.sec_molal = np.zeros(max(net.Nc, 1) * m)
        ref.iterations = np.zeros(m, np.int32)
        ref.status = np.zeros(m, np.int32)
        if self.report["train"] is not None:
            # the warm start is a per-cell function of the pre-step state:
            # predict it for the sampled cells alone
            dev = CellBatch(m)
            for f in _STATE_FIELDS + ("temperature", "saturation", "den_kg", "porosity", "volume",
                                      "soil_particle_density"):
                a = getattr(ref, f)
                if a is not None:
                    setattr(dev, f, torch.as_tensor(a, device=self.device))
            ref.alt_guess = self.step.surrogate_predict(dev).cpu().numpy()
        oracle_fn(net.as_struct(), self.opt, self.dt, ref)
        it = torch.as_tensor(idx, device=self.device)
        g = CellBatch(m)
        for f in _OUT_FIELDS:
            a = getattr(d, f)
            if a is not None:
                setattr(g, f, a.view(-1, n)[:, it].cpu().numpy().ravel().copy())
        ok = (ref.status == 0) & (g.status == 0)
        out = drift(net, g, ref, ok)
        out["cells"] = int(ok.sum())
        out["same_iterations"] = float((ref.iterations == g.iterations)[ok].mean()) if ok.any() else None
        return out
