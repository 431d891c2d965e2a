"""Batched nested-sampling engine: device buffers of many independent runs and the
iteration loop over libgbns.so.

One ``NSBatch`` holds R runs (uneven D, n, store size) in packed structure-of-arrays
buffers.  ``run()`` initialises the live points, then replays a captured CUDA graph of
``block`` iterations (each iteration = one slice-sampler shell for every active run + one
merge/register/termination kernel) until every run has terminated, and finally computes
the results (tree live-point counts, FP64 evidence statistics) on the device.

Reference correspondence (jaxns v2.6.9, src/jaxns/):
  ShardedStaticNestedSampler._run      nested_samplers/sharded/sharded_static.py:775-851
  _main_ns_thread / _collect_shell     sharded_static.py:427-574 / :210-324
  _to_results                          sharded_static.py:652-773
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np
import torch

from . import _ffi

FAMILY_MVN = 0
FAMILY_SHELLS = 1
FAMILY_LINGAUSS = 2
PRIOR_UNIFORM = 0
PRIOR_NORMAL = 1

STATUS_BITS = {1: "init rejection budget exhausted", 2: "slice shrink budget exhausted",
               4: "store full", 8: "bad parameter (uniform phase would need iterations)",
               16: "tensor-core kernel wait timed out"}

_TC_NAMES = ("ess", "evidence_uncert", "dlogZ", "max_samples", "max_num_likelihood_evaluations",
             "log_L_contour", "efficiency_threshold", "rtol", "atol", "peak_XL_frac")
_TC_FIELDS = ("ess", "evidence_uncert", "dlogZ", "max_samples", "max_nlik", "log_L_contour",
              "efficiency_threshold", "rtol", "atol", "peak_XL_frac")
_TC_FLAGS = ("has_ess", "has_evidence_uncert", "has_dlogZ", "has_max_samples", "has_max_nlik",
             "has_log_L_contour", "has_efficiency", "has_rtol", "has_atol", "has_peak_XL")


@dataclass
class RunSpec:
    """One nested-sampling run: model tables + sampler configuration (already rounded like
    ShardedStaticNestedSampler.__post_init__, sharded_static.py:625-650)."""
    D: int
    num_live_points: int
    shell_size: int
    num_slices: int
    family: int
    params: np.ndarray
    prior_kind: np.ndarray
    prior_a: np.ndarray
    prior_b: np.ndarray
    max_samples: int
    term_cond: Dict[str, float]
    key: np.ndarray
    num_phantom: int = 0
    midpoint_shrink: bool = True
    init_efficiency_threshold: float = 0.1
    store_U: bool = True
    N: int = 0
    log_L_offset: float = 0.0  # FP64 constant part of log L (device values are relative to it)
    gradient_guided: bool = False
    gradient_slice: bool = False


NCOEF_STRIDE = 16  # doubles per row of the coefficient table


def ncoef_table(nmax: int) -> np.ndarray:
    """FP64 shrinkage coefficients per live-point count n (the n-only terms of
    _update_evidence_calc_op, internals/shrinkage_statistics.py:55-73)."""
    n = np.arange(nmax + 1, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        lnn = np.log(n)
        lnn1 = np.log(n + 1.0)
        lnn2 = np.log(n + 2.0)
        T = -np.logaddexp(0.0, -lnn)
        t = -lnn1
        T2 = -np.logaddexp(0.0, np.log(2.0) - lnn)
        t2 = np.log(2.0) - lnn1 - lnn2
        tT = -np.logaddexp(0.0, -lnn) - lnn2
    out = np.zeros((nmax + 1, NCOEF_STRIDE), np.float64)
    vals = np.stack([T, t, T2, t2, tT], axis=1)
    out[:, :5] = vals
    # bytes 64-103 of a row: the same five as fp32 pairs (hi, lo), hi + lo = the FP64 value to
    # ~2^-48 relative, for the device scans that work in pair arithmetic
    hi = vals.astype(np.float32)
    with np.errstate(invalid="ignore"):
        lo = np.where(np.isfinite(hi), vals - hi.astype(np.float64), 0.0).astype(np.float32)
    pairs = np.zeros((nmax + 1, 2 * (NCOEF_STRIDE - 8)), np.float32)
    pairs[:, 0:10:2], pairs[:, 1:10:2] = hi, lo
    out[:, 8:] = pairs.view(np.float64)
    return out


def term_cond_struct(tc: Dict[str, float]) -> _ffi.TermCond:
    s = _ffi.TermCond()
    for name, field_, flag in zip(_TC_NAMES, _TC_FIELDS, _TC_FLAGS):
        v = tc.get(name)
        if v is None:
            continue
        setattr(s, flag, 1)
        setattr(s, field_, float(v))
    return s


def _dbucket(D: int) -> int:
    if D <= 8:
        return 0
    if D <= 16:
        return 1
    if D <= 32:
        return 2
    if D <= 64:
        return 3
    raise ValueError(f"D={D} > 64 is not supported by the fused slice kernel")


def param_count(family: int, D: int, N: int = 0) -> int:
    """Length of a run's parameter vector: MVN [mu, Linv, c0], shells [c1, c2, R, w, norm],
    linear-Gaussian [Phi (N x P row-major), y, sigma]."""
    if family == FAMILY_MVN:
        return D + D * D + 1
    if family == FAMILY_SHELLS:
        return 2 * D + 3
    if family == FAMILY_LINGAUSS:
        return N * D + N + 1
    raise ValueError(f"unknown likelihood family {family}")


def validate_spec(s: RunSpec, r: int = 0) -> None:
    """Reject a run the kernels would index out of bounds with (every size they read from the
    run descriptor is checked here, on the host)."""
    where = f"run {r}"
    if not 1 <= s.D <= 64:
        raise ValueError(f"{where}: D={s.D} outside [1, 64]")
    if not 1 <= s.shell_size <= s.num_live_points:
        raise ValueError(f"{where}: shell size {s.shell_size} outside [1, num_live_points={s.num_live_points}]")
    if s.num_slices < 1 or not 0 <= s.num_phantom < s.num_slices:
        raise ValueError(f"{where}: need num_slices >= 1 and 0 <= num_phantom < num_slices "
                         f"(got {s.num_slices}, {s.num_phantom})")
    if s.max_samples < 1:
        raise ValueError(f"{where}: max_samples must be positive")
    if s.family == FAMILY_LINGAUSS and s.N < 1:
        raise ValueError(f"{where}: the linear-Gaussian family needs N >= 1 data rows")
    need = param_count(s.family, s.D, s.N)
    if len(s.params) != need:
        raise ValueError(f"{where}: family {s.family} with D={s.D} takes {need} parameters, got {len(s.params)}")
    for name in ("prior_kind", "prior_a", "prior_b"):
        if len(getattr(s, name)) != s.D:
            raise ValueError(f"{where}: {name} must have D={s.D} entries")
    if not np.all(np.isin(np.asarray(s.prior_kind), (PRIOR_UNIFORM, PRIOR_NORMAL))):
        raise ValueError(f"{where}: prior kinds are {PRIOR_UNIFORM} (Uniform) or {PRIOR_NORMAL} (Normal)")
    if np.shape(s.key) != (2,):
        raise ValueError(f"{where}: key must be two uint32 words")


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    return None if t is None else t.data_ptr()


_STATE_DTYPE = np.dtype(_ffi.RunState)


class NSBatch:
    """Device state of R independent runs."""

    def __init__(self, specs: List[RunSpec], device="cuda", chains_per_item: int = 64,
                 max_evals_per_slice: int = 100000, wide_chains_per_item: int = 0, lg_tensor_cores: bool = True,
                 chains_per_lane: int = 1, warp_min_D: int = 17, lg_fused: Optional[bool] = None):
        if not specs:
            raise ValueError("no runs")
        self.specs = specs
        self.device = torch.device(device)
        R = len(specs)
        self.R = R
        dev = self.device
        Ds = np.array([s.D for s in specs])
        # 32-bit words of U storage per point: the linear-Gaussian family keeps U in FP64
        Ws = np.array([2 * s.D if s.family == FAMILY_LINGAUSS else s.D for s in specs])
        self.ucols = Ws
        ns = np.array([s.num_live_points for s in specs])
        ss = np.array([s.shell_size for s in specs])
        Ks = np.array([s.num_phantom for s in specs])
        caps = np.array([s.max_samples for s in specs], np.int64)
        if ns.max() > 4096:
            raise ValueError("at most 4096 live points per run")
        fams = {s.family for s in specs}
        self.lg = FAMILY_LINGAUSS in fams
        if self.lg and len(fams) > 1:
            raise ValueError("a batch holds either linear-Gaussian runs only or none")
        gg = {(bool(s.gradient_guided), bool(s.gradient_slice)) for s in specs}
        if len(gg) > 1:
            raise ValueError("the runs of a batch share the slice sampler's gradient options")
        self.gradient_guided, self.gradient_slice = gg.pop()
        for r, s in enumerate(specs):
            validate_spec(s, r)
        live_off = np.concatenate([[0], np.cumsum(ns)[:-1]])
        store_off = np.concatenate([[0], np.cumsum(caps)[:-1]])
        shell_off = np.concatenate([[0], np.cumsum(ss)[:-1]])
        plen = np.array([len(s.params) for s in specs])
        param_off = np.concatenate([[0], np.cumsum(plen)[:-1]])
        prior_off = np.concatenate([[0], np.cumsum(Ds)[:-1]])
        ustore = np.array([s.store_U for s in specs])
        ucap = np.where(ustore, caps * Ws, 0)
        ustore_off = np.where(ustore, np.concatenate([[0], np.cumsum(ucap)[:-1]]), -1)
        excl = lambda v: np.concatenate([[0], np.cumsum(v)[:-1]]).astype(np.int64)
        liveU_off, newU_off = excl(ns * Ws), excl(ss * Ws)
        phU_off, phL_off = excl(ss * Ks * Ws), excl(ss * Ks)
        self.offsets = dict(live=live_off, store=store_off, shell=shell_off, ustore=ustore_off, liveU=liveU_off,
                            newU=newU_off, param=param_off, phU=phU_off, phL=phL_off)

        descs = (_ffi.RunDesc * R)()
        for r, s in enumerate(specs):
            d = descs[r]
            d.D, d.n, d.s, d.S, d.K = s.D, s.num_live_points, s.shell_size, s.num_slices, s.num_phantom
            d.family, d.midpoint = s.family, int(bool(s.midpoint_shrink))
            d.uniform_phase = int(s.init_efficiency_threshold > 0.0)
            d.N = s.N
            d.ucols = int(Ws[r])
            d.init_efficiency_threshold = float(s.init_efficiency_threshold)
            d.log_L_offset = float(s.log_L_offset)
            d.cap = int(caps[r])
            d.live_off, d.store_off, d.shell_off = int(live_off[r]), int(store_off[r]), int(shell_off[r])
            d.param_off, d.prior_off, d.ustore_off = int(param_off[r]), int(prior_off[r]), int(ustore_off[r])
            d.liveU_off, d.newU_off = int(liveU_off[r]), int(newU_off[r])
            d.phU_off, d.phL_off = int(phU_off[r]), int(phL_off[r])
            d.tc = term_cond_struct(s.term_cond)
        self._descs_host = descs
        u8 = lambda obj: torch.frombuffer(bytearray(bytes(obj)), dtype=torch.uint8)
        self.t_runs = u8(descs).to(dev)
        self.t_state = torch.zeros(R * ctypes.sizeof(_ffi.RunState), dtype=torch.uint8, device=dev)
        st = (_ffi.RunState * R)()
        for r, s in enumerate(specs):
            st[r].key[0], st[r].key[1] = int(s.key[0]), int(s.key[1])
        self.t_state.copy_(u8(st))
        self.t_state0 = self.t_state.clone()
        self._state_host0 = u8(st).pin_memory() if torch.cuda.is_available() else u8(st)

        nsum, ssum, capsum = int(ns.sum()), int(ss.sum()), int(caps.sum())
        nD = int((ns * Ws).sum())
        f32, i32 = torch.float32, torch.int32
        z = lambda *shape, dtype=f32: torch.zeros(*shape, dtype=dtype, device=dev)
        self.live_U = [z(nD), z(nD)]
        self.live_L = [z(nsum), z(nsum)]
        self.live_Lc = [z(nsum), z(nsum)]
        self.live_E = [z(nsum, dtype=i32), z(nsum, dtype=i32)]
        self.live_S = [z(nsum, dtype=i32), z(nsum, dtype=i32)]
        self.new_U = z(int((ss * Ws).sum()))
        self.new_L = z(ssum)
        self.new_E = z(ssum, dtype=i32)
        self.ph_U = z(max(int((ss * Ks * Ws).sum()), 1))
        self.ph_L = z(max(int((ss * Ks).sum()), 1))
        self.store_L = torch.full((capsum,), float("inf"), dtype=f32, device=dev)
        self.store_S = z(capsum, dtype=i32)
        self.store_E = z(capsum, dtype=i32)
        self.store_P = z(capsum, dtype=torch.uint8)
        usum = int(ucap.sum())
        self.store_U = z(usum) if usum > 0 else None
        fp_host = torch.from_numpy(np.concatenate([np.asarray(s.params, np.float32) for s in specs]))
        self._fparams_host = fp_host.pin_memory() if torch.cuda.is_available() else fp_host
        self.fparams = fp_host.to(dev)
        self.prior_kind = torch.from_numpy(np.concatenate([np.asarray(s.prior_kind, np.int32) for s in specs])).to(dev)
        self.prior_a = torch.from_numpy(np.concatenate([np.asarray(s.prior_a, np.float32) for s in specs])).to(dev)
        self.prior_b = torch.from_numpy(np.concatenate([np.asarray(s.prior_b, np.float32) for s in specs])).to(dev)
        self.nmax = int(ns.max())
        # tree counts can exceed n (the sender convention of _collect_shell); cover n + 64 and
        # let the device compute larger counts' coefficients on the fly
        self.ncoef_n = self.nmax + 64
        self.ncoef = torch.from_numpy(ncoef_table(self.ncoef_n)).to(dev)

        # work items: (run, first chain, chain count), grouped by (family, D bucket),
        # longest (largest D) first inside a bucket
        CH = int(chains_per_item)
        if int(chains_per_lane) < 1:
            raise ValueError("chains_per_lane must be at least 1")
        self.chains_per_lane = int(chains_per_lane)
        items = []
        if not 2 <= int(warp_min_D) <= 17:
            raise ValueError("warp_min_D must be in [2, 17]")
        self.warp_min_D = int(warp_min_D)
        for r, s in enumerate(specs):
            if s.family == FAMILY_LINGAUSS:
                continue
            b = s.family * 4 + _dbucket(s.D)
            warp = s.family == FAMILY_MVN and s.D >= self.warp_min_D
            if warp and b < 2:
                b = 2  # a correlated Gaussian with D <= 16 on the warp-cooperative kernel (DMAX 32)
            # warp-cooperative buckets: one chain per lane of the CTA (256 lanes for D > 32,
            # 512 for D <= 32), each warp refilling its lanes from the CTA's pool
            if not warp:
                # one thread per chain, each CTA (CH lanes) drawing from a pool of
                # CH * chains_per_lane chains
                ch = CH * int(chains_per_lane)
            else:
                ch = int(wide_chains_per_item) if wide_chains_per_item else (256 if s.D > 32 else 512)
            for c0 in range(0, s.shell_size, ch):
                items.append((b, -s.D, r, c0, min(ch, s.shell_size - c0)))
        items.sort()
        arr = np.array([[it[2], it[3], it[4], 0] for it in items], np.int32).reshape(-1, 4)
        self.items = torch.from_numpy(arr if len(arr) else np.zeros((1, 4), np.int32)).to(dev)
        bb = np.full(8, 0, np.int32)
        be = np.full(8, 0, np.int32)
        bk = np.array([it[0] for it in items])
        for k in range(8):
            idx = np.nonzero(bk == k)[0]
            if len(idx):
                bb[k], be[k] = idx[0], idx[-1] + 1
        b = _ffi.Batch()
        b.num_runs, b.nmax, b.ncoef_n = R, self.nmax, self.ncoef_n
        b.runs, b.state = _ptr(self.t_runs), _ptr(self.t_state)
        for p in range(2):
            b.live_U[p], b.live_L[p], b.live_Lc[p] = _ptr(self.live_U[p]), _ptr(self.live_L[p]), _ptr(self.live_Lc[p])
            b.live_E[p], b.live_S[p] = _ptr(self.live_E[p]), _ptr(self.live_S[p])
        b.new_U, b.new_L, b.new_E = _ptr(self.new_U), _ptr(self.new_L), _ptr(self.new_E)
        b.ph_U, b.ph_L = _ptr(self.ph_U), _ptr(self.ph_L)
        b.store_L, b.store_S, b.store_E, b.store_P = (_ptr(self.store_L), _ptr(self.store_S), _ptr(self.store_E),
                                                      _ptr(self.store_P))
        b.store_U = _ptr(self.store_U)
        b.fparams, b.prior_kind, b.prior_a, b.prior_b = (_ptr(self.fparams), _ptr(self.prior_kind),
                                                         _ptr(self.prior_a), _ptr(self.prior_b))
        b.ncoef, b.items, b.num_items = _ptr(self.ncoef), _ptr(self.items), len(items)
        for k in range(8):
            b.bucket_begin[k], b.bucket_end[k] = int(bb[k]), int(be[k])
        b.chains_per_item = CH
        b.max_evals_per_slice = int(max_evals_per_slice)
        b.gradient_guided = int(self.gradient_guided)
        b.gradient_slice = int(self.gradient_slice)
        self._b = b
        self._lgb = self._alloc_lg(specs, ss, Ds, shell_off, lg_tensor_cores) if self.lg else None
        self._graphs: Dict[tuple, tuple] = {}
        self.timing = False
        self.shell_ms = 0.0
        self.shell_launch_groups = 0
        self.resid_ms = 0.0
        self.resid_launches = 0
        self.iterations_run = 0
        self.kernel_launches = 0
        self._kernels_per_iter = 1 + int(np.count_nonzero(be > bb))
        # linear-Gaussian shells: one fused launch per shell when every run's share of Phi fits in
        # the shared memory of its cluster (lg_fused=None: whenever it fits); the slice sampler's
        # gradient options run on the lock step
        self.lg_fused = False
        grads = self.gradient_guided or self.gradient_slice
        if lg_fused and grads:
            raise ValueError("the gradient options of the slice sampler run on the linear-Gaussian lock step, "
                             "not the fused shell")
        if self.lg and self.lg_tc and lg_fused is not False and not grads:
            for cs in (16, 8):
                plan = fused_plan([s.N for s in specs], int(self._lgb.pmax), (cs,))
                if plan is not None:
                    self._setup_fused(plan, ss)
                    held = ctypes.c_int(0)
                    _ffi.call("gbns_lg_fused_max_clusters", ctypes.byref(self._b), ctypes.byref(self._lgb),
                              ctypes.byref(held))
                    if held.value > 0:
                        break
                    self._teardown_fused()
            if lg_fused and not self.lg_fused:
                raise ValueError("the fused linear-Gaussian shell needs every run's rows per CTA x ceil(P / 32) "
                                 "<= 512 with clusters of 8 or 16 CTAs that the device can hold")

    def _alloc_lg(self, specs, ss, Ds, shell_off, tensor_cores=True):
        """Lock-step chain state of the linear-Gaussian family + residual work items:
        tensor cores (tcgen05, 128 chains x 256 data rows per item, proposals and Phi as
        TF32 hi/lo rows of 64 floats) or fp32 CUDA cores (64 chains x 64 rows per item)."""
        dev = self.device
        nc = int(ss.sum())
        nd = int((ss * Ds).sum())
        z = lambda n, dt=torch.float32: torch.zeros(max(n, 1), dtype=dt, device=dev)
        f64 = torch.float64
        self.lg_t = dict(j=z(nc, torch.int32), in_slice=z(nc, torch.int32), total=z(nc, torch.int32),
                         flags=z(nc, torch.int32), left=z(nc), right=z(nc), t=z(nc), alpha=z(nc), logL0=z(nc),
                         ck=z(2 * nc, torch.int32), after_key=z(2 * nc, torch.int32),
                         slices_key=z(2 * nc, torch.int32), dir_key=z(2 * nc, torch.int32), u0=z(nd), u0_lo=z(nd),
                         dir=z(nd), W=z(nd), ss=z(nc, f64), chains_left=z(len(specs), torch.int32),
                         grad=z(nd), grad_list=z(nc, torch.int64), grad_count=z(1, torch.int32))
        items = []
        for r, s in enumerate(specs):
            for c0 in range(0, s.shell_size, 64):
                for row0 in range(0, s.N, 64):
                    items.append((r, c0, min(64, s.shell_size - c0), row0))
        self.lg_items = torch.tensor(np.array(items, np.int32).reshape(-1, 4), device=dev)
        self.lg_t["chain_run"] = torch.tensor(np.repeat(np.arange(len(specs), dtype=np.int32), ss), device=dev)
        g = _ffi.LGBufs()
        for k, v in self.lg_t.items():
            setattr(g, k, v.data_ptr())
        g.items, g.num_items = self.lg_items.data_ptr(), len(items)
        g.pmax = int(max(s.D for s in specs))
        g.total_chains = nc
        if g.pmax > 64:
            raise ValueError("the linear-Gaussian path supports P <= 64")
        self.lg_tc = bool(tensor_cores)
        if self.lg_tc:
            Ns = np.array([s.N for s in specs], np.int64)
            row_base = np.concatenate([[0], np.cumsum(Ns)[:-1]]).astype(np.int64)
            rows = int(Ns.sum())
            # work units (run, 128-chain tile, first 128-row tile, row tiles): row ranges sized so
            # that there are about two units per CTA slot; the chain tiles of one row range are
            # adjacent, so the CTAs that share its Phi tiles run together
            tiles = [((s.shell_size + 127) // 128, (s.N + 127) // 128) for s in specs]
            work = sum(ct * rt for ct, rt in tiles)
            rs = max(1, min(16, work // (2 * 2 * 152)))
            items_tc = [(r, c0, rt0, min(rs, rt - rt0)) for r, (ct, rt) in enumerate(tiles)
                        for rt0 in range(0, rt, rs) for c0 in range(0, ct * 128, 128)]
            self.lg_tc_t = dict(W_hi=z(nc * 64), W_lo=z(nc * 64), Phi_hi=z(rows * 64), Phi_lo=z(rows * 64),
                                row_base=torch.tensor(row_base, device=dev),
                                items_tc=torch.tensor(np.array(items_tc, np.int32).reshape(-1, 4), device=dev))
            tile_base = np.concatenate([[0], np.cumsum([ct for ct, _ in tiles])[:-1]]).astype(np.int32)
            self.lg_tc_t.update(tile_base=torch.tensor(tile_base, device=dev),
                                tile_pending=z(sum(ct for ct, _ in tiles), torch.int32), tc_done=z(1, torch.int32))
            for k, v in self.lg_tc_t.items():
                setattr(g, k, v.data_ptr())
            g.num_tiles = int(sum(ct for ct, _ in tiles))
            g.num_items_tc = len(items_tc)
            g.total_rows = rows
            g.use_tc = 1
            _ffi.call("gbns_lg_prepare_tc", ctypes.byref(self._b), ctypes.byref(g), self._stream())
        self.lg_steps_run = 0
        return g

    def _teardown_fused(self):
        g = self._lgb
        g.items_fused, g.num_items_fused, g.cluster_size, g.rows_per_cta = None, 0, 0, 0
        self.lg_fused = False
        self._kernels_per_iter = 1

    def _setup_fused(self, plan, ss):
        cs, rows = plan
        items = [(r, c0) for r, s in enumerate(self.specs) for c0 in range(0, int(ss[r]), 128)]
        self.lg_fused_t = torch.tensor(np.array(items, np.int32).reshape(-1, 2), device=self.device)
        g = self._lgb
        g.items_fused, g.num_items_fused = self.lg_fused_t.data_ptr(), len(items)
        g.cluster_size, g.rows_per_cta = int(cs), int(rows)
        g.max_steps = int(max(s.num_slices for s in self.specs)) * 2000
        self.lg_fused = True
        self._kernels_per_iter = 2  # fused shell + merge
        self.fused_plan = {"cluster_size": int(cs), "rows_per_cta": int(rows), "clusters": len(items)}

    # ----------------------------------------------------------------- driving
    def _stream(self):
        """The current CUDA stream of the batch's device; a batch built on the CPU (layout only)
        refuses to launch anything."""
        if self.device.type != "cuda":
            raise _ffi.GBNSError(f"NSBatch on {self.device} holds host buffers; the kernels need a CUDA device "
                                 "(there is no CPU path)")
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def init(self):
        _ffi.call("gbns_batch_init", ctypes.byref(self._b), self._stream())
        self.kernel_launches += 2

    def iterate(self, k: int):
        if self.lg and self.lg_fused:
            _ffi.call("gbns_lg_iterate", ctypes.byref(self._b), ctypes.byref(self._lgb), int(k), self._stream())
            self.iterations_run += k
            self.kernel_launches += 2 * k
            return
        if self.lg:
            for _ in range(k):
                self._lg_iteration(use_graph=False)
            return
        _ffi.call("gbns_batch_iterate", ctypes.byref(self._b), int(k), self._stream())
        self.iterations_run += k
        self.kernel_launches += k * self._kernels_per_iter

    def _lg_graph(self, k: int):
        """CUDA graph of k lock-step steps; when timing, each residual launch is bracketed by
        events recorded by the graph itself."""
        key = ("lg", k, self.timing)
        ent = self._graphs.get(key)
        if ent is None:
            g = torch.cuda.CUDAGraph()
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(k)] if self.timing else []
            for a, b_ in evs:
                a.record()
                b_.record()
            torch.cuda.current_stream().synchronize()
            side = torch.cuda.Stream(device=self.device)
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.graph(g, stream=side):
                if self.timing:
                    for a, b_ in evs:
                        _ffi.call("gbns_lg_chain_step", ctypes.byref(self._b), ctypes.byref(self._lgb), self._stream())
                        _ffi.call("gbns_record_event", ctypes.c_void_p(a.cuda_event), self._stream())
                        _ffi.call("gbns_lg_residual", ctypes.byref(self._b), ctypes.byref(self._lgb), self._stream())
                        _ffi.call("gbns_record_event", ctypes.c_void_p(b_.cuda_event), self._stream())
                else:
                    _ffi.call("gbns_lg_steps", ctypes.byref(self._b), ctypes.byref(self._lgb), int(k), self._stream())
            torch.cuda.current_stream().wait_stream(side)
            ent = (g, evs)
            self._graphs[key] = ent
        return ent

    def _lg_iteration(self, use_graph: bool = True, block: int = 64):
        """One NS iteration of the linear-Gaussian batch: start the shell, advance every chain
        in blocks of `block` likelihood evaluations until all chains are done, then merge (with
        the fused shell: one launch for the shell, then the merge)."""
        if self.lg_fused:
            if use_graph:
                self.iterate_graph(1)
            else:
                _ffi.call("gbns_lg_iterate", ctypes.byref(self._b), ctypes.byref(self._lgb), 1, self._stream())
                self.iterations_run += 1
                self.kernel_launches += 2
            return
        st = self.state()
        active = (st["done"] == 0) & (st["phase"] == 1)
        if not np.any(active):
            return
        _ffi.call("gbns_lg_shell_begin", ctypes.byref(self._b), ctypes.byref(self._lgb), self._stream())
        self.kernel_launches += 1
        cap = int(max(s.num_slices for s in self.specs)) * 2000
        steps = 0
        while True:
            evs = []
            if use_graph:
                g, evs = self._lg_graph(block)
                g.replay()
            else:
                _ffi.call("gbns_lg_steps", ctypes.byref(self._b), ctypes.byref(self._lgb), int(block), self._stream())
            steps += block
            self.kernel_launches += 2 * block
            left = self.lg_t["chains_left"].cpu().numpy()
            if evs:
                self.resid_ms += sum(a.elapsed_time(b_) for a, b_ in evs)
                self.resid_launches += len(evs)
            if not np.any(left[active] > 0):
                break
            if steps > cap:
                raise _ffi.GBNSError("linear-Gaussian shell did not finish within its step budget")
        self.lg_steps_run += steps
        _ffi.call("gbns_batch_merge", ctypes.byref(self._b), self._stream())
        self.kernel_launches += 1
        self.iterations_run += 1

    def _graph(self, k: int):
        """CUDA graph of k iterations; when timing, each iteration is captured as
        [event, shell kernels, event, merge kernel] so the slice sampler's device time is
        read back from events recorded by the graph itself."""
        key = (k, self.timing)
        ent = self._graphs.get(key)
        if ent is None:
            g = torch.cuda.CUDAGraph()
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(k)] if self.timing else []
            for a, b_ in evs:  # materialise the lazily created events before capture
                a.record()
                b_.record()
            torch.cuda.current_stream().synchronize()
            side = torch.cuda.Stream(device=self.device)
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.graph(g, stream=side):
                if self.timing:
                    for a, b_ in evs:
                        _ffi.call("gbns_record_event", ctypes.c_void_p(a.cuda_event), self._stream())
                        if self.lg_fused:
                            _ffi.call("gbns_lg_shell_fused", ctypes.byref(self._b), ctypes.byref(self._lgb),
                                      self._stream())
                        else:
                            _ffi.call("gbns_batch_shell", ctypes.byref(self._b), self._stream())
                        _ffi.call("gbns_record_event", ctypes.c_void_p(b_.cuda_event), self._stream())
                        _ffi.call("gbns_batch_merge", ctypes.byref(self._b), self._stream())
                elif self.lg_fused:
                    _ffi.call("gbns_lg_iterate", ctypes.byref(self._b), ctypes.byref(self._lgb), int(k), self._stream())
                else:
                    _ffi.call("gbns_batch_iterate", ctypes.byref(self._b), int(k), self._stream())
            torch.cuda.current_stream().wait_stream(side)
            ent = (g, evs)
            self._graphs[key] = ent
        return ent

    def iterate_graph(self, k: int):
        g, evs = self._graph(k)
        g.replay()
        self.iterations_run += k
        self.kernel_launches += k * self._kernels_per_iter
        self._pending_events = evs

    def _collect_timing(self):
        evs = getattr(self, "_pending_events", None)
        if evs:
            evs[-1][1].synchronize()  # the graph's last event: every pair before it has completed
            self.shell_ms += sum(a.elapsed_time(b_) for a, b_ in evs)
            self.shell_launch_groups += len(evs)
        self._pending_events = None

    def upload_params(self):
        """Copy the likelihood parameters (MVN factors, shell centres, Phi and y) from pinned
        host memory to the device again, and re-split Phi for the tensor-core path."""
        self.fparams.copy_(self._fparams_host, non_blocking=True)
        if self.lg and self.lg_tc:
            _ffi.call("gbns_lg_prepare_tc", ctypes.byref(self._b), ctypes.byref(self._lgb), self._stream())
            self.kernel_launches += 1
        return int(self.fparams.numel() * 4)

    def reset(self, from_host: bool = False):
        """Restore every run's initial state (keys); from_host copies it from pinned memory."""
        if from_host:
            self.t_state.copy_(self._state_host0, non_blocking=True)
        else:
            self.t_state.copy_(self.t_state0)
        self.store_L.fill_(float("inf"))

    def state(self) -> np.ndarray:
        return np.frombuffer(self.t_state.cpu().numpy().tobytes(), dtype=_STATE_DTYPE)

    def all_done(self) -> bool:
        st = self.state()
        return bool(np.all(st["done"] != 0))

    def finalize(self):
        _ffi.call("gbns_batch_finalize", ctypes.byref(self._b), self._stream())
        self.kernel_launches += 1

    def run(self, block: int = 8, max_iterations: Optional[int] = None, use_graph: bool = True,
            check: bool = True) -> np.ndarray:
        """Run every run to termination; returns the final per-run state records."""
        self.init()
        if max_iterations is None:
            max_iterations = int(max(s.max_samples // max(s.shell_size, 1) + 2 for s in self.specs))
        done_it = 0
        while done_it < max_iterations:
            done = self.all_done()
            self._collect_timing()
            if done:
                break
            if self.lg and not self.lg_fused:
                self._lg_iteration(use_graph=use_graph)
                done_it += 1
                continue
            k = min(block, max_iterations - done_it)
            if use_graph:
                self.iterate_graph(k)
            else:
                self.iterate(k)
            done_it += k
        self.finalize()
        st = self.state()
        self._collect_timing()
        if not check:
            return st
        bad = st["status"] != 0
        if np.any(bad):
            r = int(np.nonzero(bad)[0][0])
            msgs = [m for bit, m in STATUS_BITS.items() if st["status"][r] & bit]
            raise _ffi.GBNSError(f"run {r}: device status {st['status'][r]} ({'; '.join(msgs)})")
        if not np.all(st["phase"] == 2):
            raise _ffi.GBNSError("iteration budget exhausted before termination")
        return st

    # ----------------------------------------------------------------- results
    def results(self, with_U: bool = True) -> Dict[str, torch.Tensor]:
        dev = self.device
        caps = np.array([s.max_samples for s in self.specs], np.int64)
        capsum = int(caps.sum())
        R = self.R
        z = lambda n, dt: torch.zeros(n, dtype=dt, device=dev)
        out = dict(samples_indices=z(capsum, torch.int32), num_live_points=z(capsum, torch.int32),
                   log_L_samples=z(capsum, torch.float64), log_dp_mean=z(capsum, torch.float64),
                   log_X_mean=z(capsum, torch.float64), nevals_sorted=z(capsum, torch.int32),
                   scalars=z(R * 8, torch.float64))
        out["U_sorted"] = z(self.store_U.numel(), torch.float32) if (with_U and self.store_U is not None) else None
        scratch_ll = z(2 * (capsum + R), torch.int64)
        scratch_i = z(capsum + R, torch.int32)
        rb = _ffi.ResultsBufs()
        rb.samples_indices, rb.num_live_points = _ptr(out["samples_indices"]), _ptr(out["num_live_points"])
        rb.log_L_samples, rb.log_dp_mean = _ptr(out["log_L_samples"]), _ptr(out["log_dp_mean"])
        rb.log_X_mean, rb.nevals_sorted = _ptr(out["log_X_mean"]), _ptr(out["nevals_sorted"])
        rb.U_sorted, rb.scalars = _ptr(out["U_sorted"]), _ptr(out["scalars"])
        rb.scratch_ll, rb.scratch_i = _ptr(scratch_ll), _ptr(scratch_i)
        _ffi.call("gbns_batch_results", ctypes.byref(self._b), ctypes.byref(rb), self._stream())
        self.kernel_launches += 1
        out["scalars"] = out["scalars"].view(R, 8)
        return out

    def run_slices(self, r: int, out: Dict[str, torch.Tensor]) -> Dict[str, torch.Tensor]:
        """Per-run views (trimmed to the run's sample count) of a results() dict."""
        st = self.state()
        s = self.specs[r]
        o = int(self.offsets["store"][r])
        N = int(min(st["num_samples"][r], s.max_samples))
        d = {k: v[o:o + N] for k, v in out.items() if k not in ("scalars", "U_sorted") and v is not None}
        if out.get("U_sorted") is not None and self.offsets["ustore"][r] >= 0:
            uo = int(self.offsets["ustore"][r])
            d["U_sorted"] = self._u_rows(out["U_sorted"][uo:uo + N * int(self.ucols[r])], r, N)
        d["scalars"] = out["scalars"][r]
        return d

    def store_view(self, r: int) -> Dict[str, torch.Tensor]:
        st = self.state()
        s = self.specs[r]
        o = int(self.offsets["store"][r])
        N = int(min(st["num_samples"][r], s.max_samples))
        raw = self.store_L[o:o + N]
        d = dict(log_L=raw.double() + s.log_L_offset, log_L_raw=raw, sender=self.store_S[o:o + N],
                 nevals=self.store_E[o:o + N], phantom=self.store_P[o:o + N])
        if self.store_U is not None and self.offsets["ustore"][r] >= 0:
            uo = int(self.offsets["ustore"][r])
            d["U"] = self._u_rows(self.store_U[uo:uo + N * int(self.ucols[r])], r, N)
        return d

    def _u_rows(self, words: torch.Tensor, r: int, rows: int) -> torch.Tensor:
        """[rows, D] view of run r's U words (float64 for the linear-Gaussian family)."""
        D = self.specs[r].D
        if self.specs[r].family == FAMILY_LINGAUSS:
            return words.view(torch.float64).view(rows, D)
        return words.view(rows, D)

    def new_U_view(self, r: int) -> torch.Tensor:
        """[s, D] view of run r's shell outputs (the chains' final points)."""
        o = int(self.offsets["newU"][r])
        s = self.specs[r].shell_size
        return self._u_rows(self.new_U[o:o + s * int(self.ucols[r])], r, s)

    def live_view(self, r: int) -> Dict[str, torch.Tensor]:
        st = self.state()
        p = int(st["parity"][r])
        s = self.specs[r]
        o = int(self.offsets["live"][r])
        uo = int(self.offsets["liveU"][r])
        n = s.num_live_points
        raw = self.live_L[p][o:o + n]
        return dict(U=self._u_rows(self.live_U[p][uo:uo + n * int(self.ucols[r])], r, n),
                    log_L=raw.double() + s.log_L_offset, log_L_raw=raw,
                    nevals=self.live_E[p][o:o + n], sender=self.live_S[p][o:o + n],
                    log_L_constraint=self.live_Lc[p][o:o + n])

    def forward(self, r: int, U: torch.Tensor) -> torch.Tensor:
        """Model.forward of run r over a batch U [B, D] (device tensor; FP64 for the
        linear-Gaussian family)."""
        if not 0 <= r < self.R:
            raise ValueError(f"run {r} out of range [0, {self.R})")
        dt = torch.float64 if self.specs[r].family == FAMILY_LINGAUSS else torch.float32
        U = U.to(device=self.device, dtype=dt).contiguous()
        if U.dim() != 2 or U.shape[1] != self.specs[r].D:
            raise ValueError(f"U must be [B, {self.specs[r].D}] for run {r}, got {tuple(U.shape)}")
        out = torch.empty(U.shape[0], dtype=torch.float32, device=self.device)
        _ffi.call("gbns_forward", ctypes.byref(self._b), int(r), ctypes.c_void_p(U.data_ptr()),
                  ctypes.c_void_p(out.data_ptr()), ctypes.c_longlong(U.shape[0]), self._stream())
        return out

    def slice_shell(self, Lstar: torch.Tensor, keys: torch.Tensor):
        """One shell of every run from the current live sets with explicit contours (relative
        to each run's log_L_offset, like the device log-likelihoods) and sample keys (test
        hook): outputs in new_U / new_L (relative) / new_E."""
        Lstar = Lstar.to(device=self.device, dtype=torch.float32).contiguous()
        keys = keys.to(device=self.device, dtype=torch.int32).contiguous()
        if Lstar.numel() != self.R or keys.numel() != 2 * self.R:
            raise ValueError(f"need one contour and one key (2 words) per run: {self.R} runs, got "
                             f"{Lstar.numel()} contours and {keys.numel()} key words")
        _ffi.call("gbns_slice_shell", ctypes.byref(self._b), ctypes.c_void_p(Lstar.data_ptr()),
                  ctypes.c_void_p(keys.data_ptr()), self._stream())

    def set_live(self, r: int, U: np.ndarray, log_L: np.ndarray):
        """Overwrite run r's current live set (test hook; values sorted, relative to the
        run's log_L_offset)."""
        st = self.state()
        p = int(st["parity"][r])
        s = self.specs[r]
        o = int(self.offsets["live"][r])
        uo = int(self.offsets["liveU"][r])
        n = s.num_live_points
        if np.shape(U) != (n, s.D) or np.shape(log_L) != (n,):
            raise ValueError(f"run {r} needs U [{n}, {s.D}] and log_L [{n}], got {np.shape(U)} and {np.shape(log_L)}")
        dt = np.float64 if s.family == FAMILY_LINGAUSS else np.float32
        words = torch.from_numpy(np.ascontiguousarray(np.asarray(U, dt).ravel()).view(np.float32))
        self.live_U[p][uo:uo + n * int(self.ucols[r])].copy_(words)
        self.live_L[p][o:o + n].copy_(torch.from_numpy(np.asarray(log_L, np.float32)))


def fused_plan(Ns, pmax: int, sizes=(16, 8)):
    """(cluster size, rows per CTA) of the fused linear-Gaussian shell, or None when a run's
    share of Phi would not fit: clusters of 16 (else 8) CTAs, each holding rows_per_cta rows
    (128, 256 or 512) of TF32 hi / lo Phi, with rows_per_cta * ceil(pmax / 32) <= 512."""
    nkb = 2 if pmax > 32 else 1
    for cs in sizes:
        need = max(128 * -(-int(N) // (cs * 128)) for N in Ns)
        rows = next((r for r in (128, 256, 512) if r >= need), None)
        if rows is not None and rows * nkb <= 512:
            return cs, rows
    return None


# --------------------------------------------------------------- model tables

def mvn_offset(cov) -> float:
    """-sum log L_ii - D/2 log 2 pi: the constant of the Gaussian log density."""
    L = np.linalg.cholesky(np.asarray(cov, np.float64))
    return float(-np.sum(np.log(np.diag(L))) - 0.5 * L.shape[0] * np.log(2.0 * np.pi))


def shells_offset(width) -> float:
    return float(-np.log(np.sqrt(2.0 * np.pi * float(width) ** 2)))


def mvn_params(mu, cov) -> np.ndarray:
    """[mu, Linv (row-major lower), c0] with L = chol(cov), c0 = -sum log L_ii - D/2 log 2 pi."""
    mu = np.asarray(mu, np.float64)
    L = np.linalg.cholesky(np.asarray(cov, np.float64))
    Linv = np.linalg.inv(L)
    Linv = np.tril(Linv)
    D = len(mu)
    c0 = -np.sum(np.log(np.diag(L))) - 0.5 * D * np.log(2.0 * np.pi)
    return np.concatenate([mu, Linv.ravel(), [c0]]).astype(np.float32)


def shells_params(c1, c2, radius, width) -> np.ndarray:
    norm = np.log(np.sqrt(2.0 * np.pi * width ** 2))
    return np.concatenate([np.asarray(c1, np.float64), np.asarray(c2, np.float64),
                           [radius, width, norm]]).astype(np.float32)
