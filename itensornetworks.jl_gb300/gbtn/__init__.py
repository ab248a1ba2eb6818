"""GB300-native belief propagation for tensor networks (host package).

Python mirror of ITensorNetworks.jl's BP interface over the C ABI of
libgbtn.so (include/gbtn.h).  Every numerical step runs on the GPU."""
from . import _lib
from ._lib import Context, GBTNError, InvalidArgument, LibraryNotBuilt, Unsupported, default_context
from .cache import (BeliefPropagationCache, default_bp_maxiter, edge_scalars, environment, expect, factors,
                    identity_messages, incoming_messages, initialize_cache,
                    inner, loginner, logscalar, message, message_diff, messages, norm, norm_sqr, normalize,
                    region_scalar, rescale, scalar, scalar_factors_quotient, update, update_factor, update_factors,
                    updated_message, vertex_scalars)
from .partition import CoarseGraining, PartitionedBPCache, partitioned_cache
from .sharded import GpuShard, ShardPlan, block_owner, run_distributed, run_local
from .su import (SimpleUpdateState, apply, bp_environments, checkerboard_edges, tebd, tebd_gates, tebd_with_pullback,
                 tfim_gate)
from .opsum import OpSum, group_terms, trotter2_gates
from .qn import QNBeliefPropagationCache, QNNetwork, random_qn_network
from .network import (TensorNetwork, default_edge_sequence, disjoint_union, parallel_edge_sequence,
                      random_network, random_tensors, square_lattice)

__all__ = [
    "BeliefPropagationCache", "Context", "GBTNError", "InvalidArgument", "LibraryNotBuilt", "TensorNetwork",
    "Unsupported", "default_context", "default_edge_sequence", "disjoint_union", "environment", "expect",
    "initialize_cache", "inner", "loginner", "logscalar", "message_diff", "norm", "norm_sqr", "normalize",
    "parallel_edge_sequence", "random_network", "random_tensors", "rescale", "scalar", "square_lattice", "update",
    "updated_message", "SimpleUpdateState", "apply", "checkerboard_edges", "tebd", "tfim_gate", "bp_environments",
    "CoarseGraining", "PartitionedBPCache", "partitioned_cache", "GpuShard", "ShardPlan", "block_owner",
    "run_distributed", "run_local", "tebd_gates", "tebd_with_pullback", "OpSum", "group_terms", "trotter2_gates",
    "edge_scalars",
    "identity_messages", "message", "messages", "update_factor", "update_factors", "vertex_scalars",
    "region_scalar", "scalar_factors_quotient", "incoming_messages", "factors", "default_bp_maxiter",
    "QNBeliefPropagationCache", "QNNetwork", "random_qn_network",
]
