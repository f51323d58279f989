"""Config and ParseParameters, mirroring lib/config.h:29-87 and
app/parse_parameters.h:30-100 of the reference.

Flags are `-key value` (value-less keys are booleans), read the way the
reference's ArgParser does (lib/tools/arg_parser.h:18-75).  `n`/`m` are log2
values unless `-exact_n`/`-exact_m` is set or the generator is grid_2d.  The
reference computes `1 << n` in int, which overflows for n >= 31
(parse_parameters.h:89); here the shift is done in 64 bits.
"""
from __future__ import annotations

from dataclasses import dataclass, field

from . import _lib


@dataclass
class Config:
    seed: int = 1
    input_type: str = "null"
    input_file: str = "null"
    output_file: str = "out"
    debug_output_file: str = "tmp"
    print_verbose: bool = False
    n: int = 0
    m: int = 0
    degree_limit: int = 100
    replicate_high_degree: bool = False
    sequential_limit: int = 1
    fixed_limit: bool = False
    iterations: int = 10
    prop_iterations: int = 3
    beta: float = 0.1
    use_bfs: bool = False
    use_regular: bool = False
    overallocate: bool = False
    use_contraction: bool = False
    direct_contraction: bool = False
    single_level_contraction: bool = False
    number_of_hitters: int = 0
    degree_threshold: int = 16
    neighborhood_sampling_factor: float = 0.5
    gen: str = "null"
    gen_n: int = 1 << 18
    gen_m: int = 1 << 18
    gen_r: float = 0.001
    gen_p: float = 1.0
    gen_periodic: bool = False
    gen_k: int = 0
    gen_gamma: float = 2.2
    gen_d: float = 16.0
    extra: dict = field(default_factory=dict)

    def to_c(self) -> _lib.cc_config:
        """The solver fields as the C ABI's cc_config."""
        c = _lib.cc_config()
        _lib.gpu().cc_config_default(c)
        c.beta = float(self.beta)
        c.seq = int(self.sequential_limit)
        c.prop_iterations = int(self.prop_iterations)
        c.number_of_hitters = int(self.number_of_hitters)
        c.degree_threshold = int(self.degree_threshold)
        c.degree_limit = int(self.degree_limit)
        c.hd_sf = float(self.neighborhood_sampling_factor)
        c.fixed_seq = int(self.fixed_limit)
        c.contraction = int(self.use_contraction)
        c.direct = int(self.direct_contraction)
        c.single = int(self.single_level_contraction)
        c.bfs = int(self.use_bfs)
        c.replicate = int(self.replicate_high_degree)
        c.regular = int(self.use_regular)
        c.overalloc = int(self.overallocate)
        c.verbose = int(self.print_verbose)
        return c


class ArgParser:
    """ArgParser (lib/tools/arg_parser.h:21-38): every token that starts with
    '-' is a key; the next token is its value unless it also starts with '-'.
    A key without a value is a set flag whose value is the empty string; a
    numeric Get of it yields 0, as a failed istringstream extraction does."""

    def __init__(self, argv: list[str]):
        self.kv: dict[str, str] = {}
        self.data: list[str] = []
        i = 0
        while i < len(argv):
            a = argv[i]
            if a.startswith("-"):
                key = a[1:]
                i += 1
                if i < len(argv) and not argv[i].startswith("-"):
                    self.kv[key] = argv[i]
                    i += 1
                else:
                    self.kv[key] = ""
            else:
                self.data.append(a)
                i += 1

    def is_set(self, key: str) -> bool:
        return key in self.kv

    def get(self, key: str, default, typ=None):
        if key not in self.kv:
            return default
        t = typ or type(default)
        s = self.kv[key]
        if t is str:
            return s
        try:
            return t(s)
        except ValueError:
            return t(0)


def parse_parameters(argv: list[str], conf: Config | None = None) -> Config:
    """ParseParameters (app/parse_parameters.h:30-100)."""
    a = ArgParser(argv)
    c = conf or Config()
    c.seed = a.get("seed", 1, int)
    c.input_type = a.get("input", "null", str)
    c.input_file = a.get("in", "null", str)
    c.output_file = a.get("out", "out", str)
    c.debug_output_file = a.get("debug_out", "tmp", str)
    c.print_verbose = a.is_set("verbose")
    c.iterations = a.get("i", 10, int)
    c.prop_iterations = a.get("pi", 3, int)
    c.number_of_hitters = a.get("heavy-hitters", 0, int)
    c.beta = a.get("beta", 0.1, float)
    c.use_contraction = a.is_set("contraction")
    c.direct_contraction = a.is_set("direct")
    c.single_level_contraction = a.is_set("single")
    c.sequential_limit = a.get("seq", 1, int)
    c.fixed_limit = a.is_set("fixed-seq")
    c.degree_limit = a.get("deg", 100, int)
    c.degree_threshold = a.get("hd-thres", 16, int)
    c.neighborhood_sampling_factor = a.get("hd-sf", 0.5, float)
    c.replicate_high_degree = a.is_set("replicate")
    c.use_bfs = a.is_set("bfs")
    c.use_regular = a.is_set("regular")
    c.overallocate = a.is_set("overalloc")
    c.gen = a.get("gen", "null", str)
    c.gen_k = a.get("k", 0, int)
    exact_n = a.is_set("exact_n") or c.gen == "grid_2d"
    c.gen_n = a.get("n", 18, int) if exact_n else (1 << a.get("n", 18, int))
    exact_m = a.is_set("exact_m") or c.gen == "grid_2d"
    c.gen_m = a.get("m", 18, int) if exact_m else (1 << a.get("m", 18, int))
    c.gen_r = a.get("r", 0.001, float)
    c.gen_gamma = a.get("gamma", 2.2, float)
    c.gen_d = a.get("d", 16.0, float)
    c.gen_p = a.get("p", 1.0, float)
    c.gen_periodic = a.is_set("periodic")
    return c
