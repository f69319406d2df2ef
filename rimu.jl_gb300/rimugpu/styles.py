"""StochasticStyle traits (src/StochasticStyles/styles.jl) and their step parameters."""
from __future__ import annotations

import math

from . import _lib


class NoCompression:
    def __repr__(self):
        return "NoCompression()"


class ThresholdCompression:
    """ThresholdCompression(threshold=1) (compression.jl:8-11)."""

    def __init__(self, threshold=1.0):
        self.threshold = float(threshold)

    def __repr__(self):
        return f"ThresholdCompression({self.threshold})"


class WithReplacement:
    """WithReplacement(threshold=0) (spawning.jl:226-230)."""

    def __init__(self, threshold=0.0):
        self.threshold = float(threshold)


class Exact:
    def __init__(self, threshold=0.0):
        self.threshold = float(threshold)


class StochasticStyle:
    code = -1
    valtype = float
    compression = NoCompression()

    def step_stat_names(self) -> tuple:
        raise NotImplementedError

    def compression_names(self) -> tuple:
        return ("len_before",) if isinstance(self.compression, ThresholdCompression) else ()

    def params(self) -> dict:
        return dict(style=self.code, proj_threshold=0.0, compression=0.0,
                    rel_spawning_threshold=1.0, abs_spawning_threshold=math.inf)


class IsStochasticInteger(StochasticStyle):
    """Integer walkers (styles.jl:11-25); spawning WithReplacement, stochastic rounding."""
    code = _lib.STYLE_INTEGER
    valtype = int

    def step_stat_names(self):
        return ("spawn_attempts", "spawns", "deaths", "clones", "zombies")

    def __repr__(self):
        return "IsStochasticInteger{Int64}()"


class IsDeterministic(StochasticStyle):
    """Deterministic multiplication (styles.jl:76-105), optional compression."""
    code = _lib.STYLE_DETERMINISTIC
    valtype = float

    def __init__(self, compression=None):
        self.compression = compression if compression is not None else NoCompression()

    def step_stat_names(self):
        return ("exact_steps",)

    def params(self):
        p = super().params()
        if isinstance(self.compression, ThresholdCompression):
            p["compression"] = self.compression.threshold
        return p

    def __repr__(self):
        return f"IsDeterministic{{Float64}}({self.compression})"


class IsDynamicSemistochastic(StochasticStyle):
    """IsDynamicSemistochastic (styles.jl:175-214) with WithReplacement sub-strategy."""
    code = _lib.STYLE_DSS
    valtype = float

    def __init__(self, threshold=1.0, rel_spawning_threshold=1.0,
                 abs_spawning_threshold=math.inf, late_compression=True, compression=None,
                 spawning=None):
        if compression is None:
            compression = ThresholdCompression(threshold) if late_compression else NoCompression()
        if spawning is None:
            spawning = WithReplacement() if late_compression else WithReplacement(threshold)
        if not isinstance(spawning, WithReplacement):
            raise ValueError("only the WithReplacement spawning strategy runs on the GPU")
        self.compression = compression
        self.spawning = spawning
        self.proj_threshold = float(spawning.threshold)
        self.rel_spawning_threshold = float(rel_spawning_threshold)
        self.abs_spawning_threshold = float(abs_spawning_threshold)

    def step_stat_names(self):
        return ("exact_steps", "inexact_steps", "spawn_attempts", "spawns")

    def params(self):
        p = super().params()
        p.update(proj_threshold=self.proj_threshold,
                 rel_spawning_threshold=self.rel_spawning_threshold,
                 abs_spawning_threshold=self.abs_spawning_threshold)
        if isinstance(self.compression, ThresholdCompression):
            p["compression"] = self.compression.threshold
        return p

    def __repr__(self):
        return "IsDynamicSemistochastic{Float64,%s,DynamicSemistochastic}()" % type(
            self.compression).__name__


def default_style(valtype):
    """default_style (styles.jl:216-219)."""
    return IsStochasticInteger() if valtype is int else IsDeterministic()
