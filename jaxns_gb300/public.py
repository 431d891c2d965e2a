"""jaxns-compatible public API: TerminationCondition, samplers, ShardedStaticNestedSampler
and NestedSampler / DefaultNestedSampler, driving the sm_103a kernels of libgbns.so.

Reference: jaxns v2.6.9 public.py:30-222, nested_samplers/sharded/sharded_static.py:577-851,
samplers/uni_slice_sampler.py:276-441, samplers/uniform_samplers.py:21-85,
nested_samplers/common/types.py.
"""
from __future__ import annotations

import dataclasses
import warnings
from typing import Any, List, NamedTuple, Optional, Union

import numpy as np
import torch

from .engine import NSBatch, RunSpec
from .framework import Model

__all__ = ["TerminationCondition", "NestedSamplerResults", "NestedSampler", "DefaultNestedSampler",
           "UniDimSliceSampler", "UniformSampler", "ShardedStaticNestedSampler", "NestedSamplerState",
           "SampleCollection", "round_up_num_live_points", "round_up_max_samples"]

INT64_MAX = float(np.iinfo(np.int64).max)


class TerminationCondition(NamedTuple):
    """nested_samplers/common/types.py:26-60 (same fields and bit meanings)."""
    ess: Optional[float] = None
    evidence_uncert: Optional[float] = None
    live_evidence_frac: Optional[float] = None
    dlogZ: Optional[float] = None
    max_samples: Optional[float] = None
    max_num_likelihood_evaluations: Optional[float] = None
    log_L_contour: Optional[float] = None
    efficiency_threshold: Optional[float] = None
    rtol: Optional[float] = None
    atol: Optional[float] = None
    peak_XL_frac: Optional[float] = None

    def __and__(self, other):
        return TerminationConditionConjunction(conds=[self, other])

    def __or__(self, other):
        return TerminationConditionDisjunction(conds=[self, other])

    def as_dict(self):
        if self.live_evidence_frac is not None:
            warnings.warn("live_evidence_frac is deprecated, use dlogZ instead.")
        d = {k: (None if v is None else float(v)) for k, v in self._asdict().items()}
        d.pop("live_evidence_frac")
        return d


class TerminationConditionConjunction(NamedTuple):
    conds: list


class TerminationConditionDisjunction(NamedTuple):
    conds: list


class NestedSamplerResults(NamedTuple):
    """nested_samplers/common/types.py:77-98."""
    log_Z_mean: float
    log_Z_uncert: float
    ESS: float
    H_mean: float
    samples: dict
    parametrised_samples: dict
    U_samples: Any
    log_L_samples: Any
    log_dp_mean: Any
    log_X_mean: Any
    log_posterior_density: Any
    num_live_points_per_sample: Any
    num_likelihood_evaluations_per_sample: Any
    total_num_samples: int
    total_phantom_samples: int
    total_num_likelihood_evaluations: int
    log_efficiency: float
    termination_reason: int


class SampleCollection(NamedTuple):
    sender_node_idx: Any
    log_L: Any
    U_samples: Any
    num_likelihood_evaluations: Any
    phantom: Any


class NestedSamplerState(NamedTuple):
    key: np.ndarray
    next_sample_idx: int
    num_samples: int
    sample_collection: SampleCollection
    batch: Any = None   # device-resident engine state (NSBatch) and run index
    run: int = 0


def round_up_num_live_points(init_num_live_points, shell_frac, num_devices):
    """sharded_static.py:577-584"""
    n = int(init_num_live_points)
    while int(n * shell_frac) % num_devices != 0:
        n += 1
    return n


def round_up_max_samples(init_max_samples, num_discard, num_phantom_points):
    """sharded_static.py:587-594"""
    m = int(init_max_samples)
    block = num_discard * (1 + num_phantom_points)
    while m % block != 0:
        m += 1
    return m


@dataclasses.dataclass(eq=False)
class UniDimSliceSampler:
    """samplers/uni_slice_sampler.py:276-326 (configuration and validation); the chain
    itself runs in the fused kernel of gbns_slice.cu."""
    model: Model
    num_slices: int
    num_phantom_save: int
    midpoint_shrink: bool
    perfect: bool
    gradient_slice: bool = False
    adaptive_shrink: bool = False
    gradient_guided: bool = False

    def __post_init__(self):
        if self.num_slices < 1:
            raise ValueError(f"num_slices should be >= 1, got {self.num_slices}.")
        if self.num_phantom_save < 0:
            raise ValueError(f"num_phantom_save should be >= 0, got {self.num_phantom_save}.")
        if self.num_phantom_save >= self.num_slices:
            raise ValueError(
                f"num_phantom_save should be < num_slices, got {self.num_phantom_save} >= {self.num_slices}.")
        self.num_slices = int(self.num_slices)
        self.num_phantom_save = int(self.num_phantom_save)
        if self.adaptive_shrink:
            raise NotImplementedError("Adaptive shrinkage not implemented.")
        if not self.perfect:
            raise ValueError("Only perfect slice sampler is implemented.")
        self.gradient_slice = bool(self.gradient_slice)

    def num_phantom(self) -> int:
        return self.num_phantom_save


@dataclasses.dataclass(eq=False)
class UniformSampler:
    """samplers/uniform_samplers.py:21-40."""
    model: Model
    max_likelihood_evals: int = 100

    def __post_init__(self):
        if self.max_likelihood_evals < 1:
            raise ValueError("max_likelihood_evals must be >= 1")

    def num_phantom(self) -> int:
        return 0


@dataclasses.dataclass(eq=False)
class ShardedStaticNestedSampler:
    """sharded_static.py:597-851 on one GPU (the 'shard' mesh has a single device)."""
    model: Model
    max_samples: int
    init_efficiency_threshold: float
    sampler: UniDimSliceSampler
    num_live_points: int
    shell_fraction: Optional[float] = None
    num_dynamic_refinement_iterations: int = 0
    refine_threshold: float = 0.01
    devices: Optional[List[Any]] = None
    verbose: bool = False
    store_U: bool = True

    def __post_init__(self):
        if self.shell_fraction is None:
            self.shell_fraction = 0.5
        self.shell_fraction = max(self.shell_fraction, 1. / self.num_live_points)
        if (self.shell_fraction <= 0.) or (self.shell_fraction > 1.):
            raise ValueError(
                f"Expected 0 < shell_fraction <= 1, got {self.shell_fraction}. Best to keep it around 0.5.")
        if self.num_dynamic_refinement_iterations > 0:
            raise NotImplementedError("dynamic refinement is not on the GPU path")
        self.num_live_points = round_up_num_live_points(self.num_live_points, self.shell_fraction, 1)
        self.max_samples = round_up_max_samples(self.max_samples, int(self.shell_fraction * self.num_live_points),
                                                self.sampler.num_phantom())

    def run_spec(self, key, term_cond: TerminationCondition) -> RunSpec:
        m = self.model
        return RunSpec(D=m.U_ndims, num_live_points=self.num_live_points,
                       shell_size=int(self.num_live_points * self.shell_fraction),
                       num_slices=self.sampler.num_slices, family=m.family, params=m.family_params(),
                       prior_kind=m.prior_kind, prior_a=m.prior_a, prior_b=m.prior_b,
                       max_samples=self.max_samples, term_cond=term_cond.as_dict(), key=np.asarray(key, np.uint32),
                       num_phantom=self.sampler.num_phantom(), midpoint_shrink=self.sampler.midpoint_shrink,
                       init_efficiency_threshold=self.init_efficiency_threshold, store_U=self.store_U,
                       N=int(getattr(m.log_likelihood, "Phi", np.zeros((0, 0))).shape[0]),
                       log_L_offset=m.log_likelihood.log_L_offset(),
                       gradient_guided=bool(getattr(self.sampler, "gradient_guided", False)),
                       gradient_slice=bool(getattr(self.sampler, "gradient_slice", False)))

    def _run(self, key, term_cond: TerminationCondition):
        batch = NSBatch([self.run_spec(key, term_cond)], device="cuda")
        st = batch.run()
        return int(st["termination_reason"][0]), batch

    def _to_results(self, termination_reason, state: NestedSamplerState, trim: bool = True) -> NestedSamplerResults:
        return results_from_batch(self.model, state.batch, state.run, termination_reason)


def results_from_batch(model: Model, batch: NSBatch, r: int, termination_reason: int) -> NestedSamplerResults:
    out = batch.results(with_U=True)
    v = batch.run_slices(r, out)
    sc = v["scalars"].cpu().numpy()
    U = v.get("U_sorted")
    if U is not None:
        X, lpd = model.transform_device(U, log_L=v["log_L_samples"])
        samples = model.unflatten(X)
    else:
        samples, lpd = {}, None
    return NestedSamplerResults(
        log_Z_mean=float(sc[0]), log_Z_uncert=float(sc[1]), ESS=float(sc[2]), H_mean=float(sc[3]),
        samples=samples, parametrised_samples=samples, U_samples=U, log_L_samples=v["log_L_samples"],
        log_dp_mean=v["log_dp_mean"], log_X_mean=v["log_X_mean"], log_posterior_density=lpd,
        num_live_points_per_sample=v["num_live_points"].long(),
        num_likelihood_evaluations_per_sample=v["nevals_sorted"].long(), total_num_samples=int(sc[4]),
        total_phantom_samples=int(sc[5]), total_num_likelihood_evaluations=int(sc[6]),
        log_efficiency=float(sc[7]), termination_reason=int(termination_reason))


@dataclasses.dataclass(eq=False)
class NestedSampler:
    """public.py:30-222: the phantom-powered static nested sampler with the same defaults
    (s=5, k=0, c=30*D, max_samples=100*c*(k+1), num_slices=s*D)."""
    model: Model
    max_samples: Optional[Union[int, float]] = None
    num_live_points: Optional[int] = None
    num_slices: Optional[int] = None
    s: Optional[Union[int, float]] = None
    k: Optional[int] = None
    c: Optional[int] = None
    devices: Optional[List[Any]] = None
    difficult_model: bool = False
    parameter_estimation: bool = False
    shell_fraction: float = 0.5
    gradient_guided: bool = False
    init_efficiency_threshold: float = 0.1
    verbose: bool = False
    store_U: bool = True

    def __post_init__(self):
        if self.num_slices is None:
            if self.difficult_model:
                self.s = 10 if self.s is None else float(self.s)
            else:
                self.s = 5 if self.s is None else float(self.s)
            if self.s <= 0:
                raise ValueError(f"Expected s > 0, got s={self.s}")
            self.num_slices = self.model.U_ndims * self.s
        self.num_slices = int(self.num_slices)
        if self.parameter_estimation:
            s = self.s if self.s is not None else 5
            max_k = s * self.model.U_ndims - 1
            self.k = min(self.model.U_ndims, max_k) if self.k is None else int(self.k)
        else:
            self.k = 0 if self.k is None else int(self.k)
        if not (0 <= self.k < self.num_slices):
            raise ValueError(f"Expected 0 <= k < num_slices, got k={self.k}, num_slices={self.num_slices}, "
                             f"U_ndims={self.model.U_ndims}")
        if self.num_live_points is not None:
            self.c = max(1, int(self.num_live_points / (self.k + 1)))
        else:
            if self.difficult_model:
                self.c = 100 * self.model.U_ndims if self.c is None else int(self.c)
            else:
                self.c = 30 * self.model.U_ndims if self.c is None else int(self.c)
            if self.c <= 0:
                raise ValueError(f"Expected c > 0, got c={self.c}")
        if self.max_samples is None:
            self.max_samples = self.c * (self.k + 1) * 100
        self.max_samples = int(self.max_samples)
        self._nested_sampler = ShardedStaticNestedSampler(
            model=self.model, num_live_points=self.c, max_samples=self.max_samples,
            sampler=UniDimSliceSampler(model=self.model, num_slices=self.num_slices, num_phantom_save=self.k,
                                       midpoint_shrink=not self.difficult_model,
                                       gradient_guided=self.gradient_guided, perfect=True),
            init_efficiency_threshold=self.init_efficiency_threshold, shell_fraction=self.shell_fraction,
            devices=self.devices, verbose=self.verbose, store_U=self.store_U)
        self.num_live_points = self._nested_sampler.num_live_points
        # post-analysis utilities attached as in the reference (summary and plotting are not built)
        from .utils import load_results, save_results
        self.save_results = save_results
        self.load_results = load_results

    @property
    def nested_sampler(self) -> ShardedStaticNestedSampler:
        return self._nested_sampler

    def normalise_term_cond(self, term_cond: Optional[TerminationCondition]) -> TerminationCondition:
        """public.py:153-170"""
        if term_cond is None:
            if self.parameter_estimation:
                term_cond = TerminationCondition(peak_XL_frac=0.1, max_samples=INT64_MAX)
            else:
                term_cond = TerminationCondition(dlogZ=float(np.log(1. + 1e-3)), max_samples=INT64_MAX)
        if not isinstance(term_cond, TerminationCondition):
            raise TypeError("NestedSampler accepts a single TerminationCondition (the reference replaces "
                            "its max_samples field, which conjunctions/disjunctions do not have)")
        return term_cond._replace(max_samples=(min(float(term_cond.max_samples), float(self._nested_sampler.max_samples))
                                               if term_cond.max_samples is not None
                                               else float(self._nested_sampler.max_samples)))

    def __call__(self, key, term_cond: Optional[TerminationCondition] = None):
        term_cond = self.normalise_term_cond(term_cond)
        reason, batch = self._nested_sampler._run(key, term_cond)
        return reason, state_from_batch(batch, 0)

    def to_results(self, termination_reason, state: NestedSamplerState, trim: bool = True) -> NestedSamplerResults:
        """public.py:177-196.  The per-sample arrays always hold exactly the run's samples (the
        device results pass reads the run's own slice of the store), so ``trim`` changes nothing;
        it is accepted for the reference's signature."""
        return self._nested_sampler._to_results(termination_reason, state, trim)

    @staticmethod
    def trim_results(results: NestedSamplerResults) -> NestedSamplerResults:
        """public.py:198-220: every array of more than one element, also inside the ``samples``
        dicts, cut to its first ``results.total_num_samples`` rows; scalars unchanged."""
        n = int(results.total_num_samples)

        def size(x):
            return x.numel() if hasattr(x, "numel") else int(np.size(x))

        def trim(x):
            if isinstance(x, dict):
                return {k: trim(v) for k, v in x.items()}
            if hasattr(x, "shape") and len(x.shape) > 0 and size(x) > 1:
                return x[:n]
            return x

        return results._replace(**{f: trim(getattr(results, f)) for f in results._fields})


def state_from_batch(batch: NSBatch, r: int) -> NestedSamplerState:
    st = batch.state()[r]
    v = batch.store_view(r)
    sc = SampleCollection(sender_node_idx=v["sender"], log_L=v["log_L"], U_samples=v.get("U"),
                          num_likelihood_evaluations=v["nevals"], phantom=v["phantom"])
    return NestedSamplerState(key=np.array(st["key"], np.uint32), next_sample_idx=int(st["next_sample_idx"]),
                              num_samples=int(st["num_samples"]), sample_collection=sc, batch=batch, run=r)


DefaultNestedSampler = NestedSampler
