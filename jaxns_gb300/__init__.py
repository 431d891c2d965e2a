"""jaxns_gb300 -- jaxns's nested-sampling inner loop on one GB300 (sm_103a).

Drop-in names: Model, Prior, NestedSampler / DefaultNestedSampler, TerminationCondition,
NestedSamplerResults.  Compute runs in libgbns.so (hand-written CUDA); there is no CPU path.
"""
from .framework import Model, Prior, Uniform, Normal, MultivariateNormalTriL, InvalidPriorName
from .likelihoods import MultivariateNormalLikelihood, GaussianShellsLikelihood, LinearGaussianLikelihood
from .public import (TerminationCondition, NestedSamplerResults, NestedSampler, DefaultNestedSampler,
                     UniDimSliceSampler, UniformSampler, ShardedStaticNestedSampler, NestedSamplerState,
                     round_up_num_live_points, round_up_max_samples)
from . import random
from .utils import sample_evidence, save_results, load_results, save_pytree, load_pytree

__version__ = "0.1.0"
