"""Numerical configuration (the YAML file given with ``--nc``).

Restates ``src/Formura/NumericalConfig.hs``:

* user-facing keys and their validation: ``NumericalConfig.hs:24-64``
  (``length_per_node``, ``grid_per_node``, ``grid_per_block``,
  ``temporal_blocking_interval``, ``filter_interval``, ``mpi_shape``,
  ``with_omp``);
* conversion to the internal configuration, blocking type and the
  divisibility rule ``(N + 2*s*nt) mod grid_per_block == 0``:
  ``NumericalConfig.hs:111-143``.

PyYAML is not a dependency: the configuration files are flat ``key: value``
maps whose values are numbers or ``[a, b, c]`` lists, so a small reader for
that subset lives here.  Keys under ``gpu_`` are backend extensions (fused
step depth, tile shape, precision) and are ignored by the reference.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from fractions import Fraction
from typing import Dict, List, Optional


class ConfigError(ValueError):
    """Raised for configurations the reference rejects (``ConfigException``)."""


def _parse_scalar(tok: str):
    tok = tok.strip()
    if not tok:
        raise ConfigError("empty value")
    try:
        return int(tok)
    except ValueError:
        pass
    try:
        # keep decimal literals exact, like Data.Scientific does
        return Fraction(tok)
    except ValueError:
        pass
    if (tok[0] == tok[-1]) and tok[0] in "'\"":
        return tok[1:-1]
    return tok


def read_yaml_subset(text: str) -> Dict[str, object]:
    """Read ``key: value`` lines; values are scalars or flow lists ``[..]``."""
    out: Dict[str, object] = {}
    for lineno, raw in enumerate(text.splitlines(), 1):
        line = raw.split("#", 1)[0].rstrip()
        if not line.strip():
            continue
        if ":" not in line:
            raise ConfigError(f"line {lineno}: expected 'key: value'")
        key, val = line.split(":", 1)
        key = key.strip()
        val = val.strip()
        if val.startswith("["):
            if not val.endswith("]"):
                raise ConfigError(f"line {lineno}: unterminated list")
            body = val[1:-1].strip()
            out[key] = [] if not body else [_parse_scalar(t) for t in body.split(",")]
        else:
            out[key] = _parse_scalar(val)
    return out


@dataclass
class NumericalConfig:
    """User configuration, ``NumericalConfig.hs:24-32``."""
    length_per_node: List[Fraction]
    grid_per_node: List[int]
    grid_per_block: Optional[List[int]] = None
    temporal_blocking_interval: Optional[int] = None
    filter_interval: Optional[int] = None
    mpi_shape: Optional[List[int]] = None
    with_omp: Optional[int] = None
    gpu: Dict[str, object] = field(default_factory=dict)


_KNOWN = ("length_per_node", "grid_per_node", "grid_per_block",
          "temporal_blocking_interval", "filter_interval", "mpi_shape", "with_omp")


def decode_config(text: str) -> NumericalConfig:
    """``decodeConfig`` (``NumericalConfig.hs:52-64``): decode and validate."""
    d = read_yaml_subset(text)
    for req in ("length_per_node", "grid_per_node"):
        if req not in d:
            raise ConfigError(f"missing required key: {req}")
    gpu = {k: v for k, v in d.items() if k.startswith("gpu_")}
    unknown = [k for k in d if k not in _KNOWN and not k.startswith("gpu_")]
    if unknown:
        raise ConfigError(f"unknown keys: {unknown}")

    def lst(k, conv):
        v = d.get(k)
        if v is None:
            return None
        if not isinstance(v, list):
            raise ConfigError(f"{k} should be a list")
        return [conv(x) for x in v]

    def num(x):
        if isinstance(x, str):
            raise ConfigError(f"not a number: {x}")
        return Fraction(x)

    def integer(x):
        if isinstance(x, int):
            return x
        if isinstance(x, Fraction) and x.denominator == 1:
            return int(x)
        raise ConfigError(f"not an integer: {x}")

    def opt_int(k):
        v = d.get(k)
        return None if v is None else integer(v)

    cfg = NumericalConfig(
        length_per_node=lst("length_per_node", num),
        grid_per_node=lst("grid_per_node", integer),
        grid_per_block=lst("grid_per_block", integer),
        temporal_blocking_interval=opt_int("temporal_blocking_interval"),
        filter_interval=opt_int("filter_interval"),
        mpi_shape=lst("mpi_shape", integer),
        with_omp=opt_int("with_omp"),
        gpu=gpu,
    )
    if not cfg.length_per_node:
        raise ConfigError("length_per_node should be a nonempty list")
    if not cfg.grid_per_node:
        raise ConfigError("grid_per_node should be a nonempty list")
    if cfg.grid_per_block is not None and not cfg.grid_per_block:
        raise ConfigError("grid_per_block should be a nonempty list")
    if cfg.mpi_shape is not None and not cfg.mpi_shape:
        raise ConfigError("mpi_shape should be a nonempty list")
    if cfg.temporal_blocking_interval is not None and cfg.temporal_blocking_interval < 1:
        raise ConfigError("temporal_blocking_interval should be a positive integer")
    if cfg.filter_interval is not None and cfg.filter_interval < 1:
        raise ConfigError("filter_interval should be a positive integer")
    if cfg.with_omp is not None and cfg.with_omp not in (0, 1, 2):
        raise ConfigError("with_omp should be 0, 1 or 2")
    return cfg


def read_config(path: str) -> NumericalConfig:
    with open(path) as f:
        return decode_config(f.read())


@dataclass
class Blocking:
    """``BlockingType`` (``NumericalConfig.hs:74-80``); ``nt == 1`` and no
    blocks means NoBlocking."""
    temporal: bool
    grid_per_block: List[int] = field(default_factory=list)
    block_per_node: List[int] = field(default_factory=list)
    nt: int = 1


@dataclass
class InternalConfig:
    """``InternalConfig`` (``NumericalConfig.hs:82-93``)."""
    length_per_node: List[Fraction]
    grid_per_node: List[int]
    space_interval: List[float]
    blocking: Blocking
    sleeve: int
    sleeve0: Optional[int]
    filter_sleeve: Optional[int]
    filter_interval: Optional[int]
    mpi_shape: Optional[List[int]]
    with_omp: int
    gpu: Dict[str, object]


def convert_config(s: int, s0: Optional[int], sf: Optional[int],
                   nc: NumericalConfig) -> InternalConfig:
    """``convertConfig`` (``NumericalConfig.hs:111-143``)."""
    nt = nc.temporal_blocking_interval if nc.temporal_blocking_interval else 1
    total = [n + 2 * s * nt for n in nc.grid_per_node]
    if nc.grid_per_block is not None and nc.temporal_blocking_interval is not None:
        gpb = list(nc.grid_per_block)
        bpn = [t // g for t, g in zip(total, gpb)]
        blocking = Blocking(True, gpb, bpn, nc.temporal_blocking_interval)
    else:
        blocking = Blocking(False)
    ms = None
    if nc.grid_per_block is not None:
        ms = [t % g for t, g in zip(total, nc.grid_per_block)]
    ic = InternalConfig(
        length_per_node=list(nc.length_per_node),
        grid_per_node=list(nc.grid_per_node),
        space_interval=[float(l) / float(n) for l, n in zip(nc.length_per_node, nc.grid_per_node)],
        blocking=blocking,
        sleeve=s, sleeve0=s0, filter_sleeve=sf,
        filter_interval=nc.filter_interval,
        mpi_shape=list(nc.mpi_shape) if nc.mpi_shape is not None else None,
        with_omp=nc.with_omp if nc.with_omp is not None else 0,
        gpu=dict(nc.gpu),
    )
    if any(l < 0 for l in ic.length_per_node):
        raise ConfigError("the element of length_per_node should be a positive number")
    if any(n < 1 for n in ic.grid_per_node):
        raise ConfigError("the element of grid_per_node should be a positive integer")
    if ic.mpi_shape is not None and any(m < 1 for m in ic.mpi_shape):
        raise ConfigError("the element of mpi_shape should be a positive integer")
    if ic.filter_interval is not None and ic.filter_interval % nt != 0:
        raise ConfigError("the filter interval is a multiple of temporal blocking interval")
    if ms is not None and any(m != 0 for m in ms):
        raise ConfigError("Inconsistent config")
    return ic
