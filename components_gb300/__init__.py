"""components_gb300: the connected-components hot path of sebalamm/components,
built for one GB300 (sm_103a).

Native parts (built in-tree by components_gb300.build):
  _build/libccgpu.so  CUDA kernels and the C ABI of include/cc_gpu.h
  _build/libccgen.so  seeded synthetic graph generators (include/cc_gen.h)
"""
from .config import Config, parse_parameters
from .graph import (StaticGraph, from_edges, gen_gnm, gen_gnm_device, gen_grid, gen_grid_device,
                    gen_rhg, gen_rhg_device, load_graph, read_binary_edges, read_binary_edges_device,
                    read_edge_list, read_metis, read_metis_device)
from .solvers import (AllReduce, Context, ExponentialContraction, LocalContraction, Propagation,
                      ShortcutPropagation, SOLVERS, component_sizes, find_components)

__all__ = ["Config", "parse_parameters", "StaticGraph", "from_edges", "gen_gnm", "gen_gnm_device",
           "gen_grid", "gen_grid_device", "load_graph", "read_binary_edges", "read_edge_list",
           "gen_rhg", "gen_rhg_device", "read_metis", "read_metis_device", "read_binary_edges_device",
           "AllReduce", "Context", "ExponentialContraction", "LocalContraction", "Propagation", "ShortcutPropagation", "SOLVERS", "component_sizes",
           "find_components"]
