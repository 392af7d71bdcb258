"""Numerical config decoding and conversion.

The decode cases restate the reference's own unit tests
(test/NumericalConfigSpec.hs:11-86): three valid decodes, three invalid
ones; the conversion cases follow NumericalConfig.hs:111-143.
"""
from fractions import Fraction

import pytest

from formura_gb300.generator.config import ConfigError, convert_config, decode_config


def test_1d_temporal_blocking():
    c = decode_config("length_per_node: [1.0]\ngrid_per_node: [10]\ngrid_per_block: [10]\n"
                      "mpi_shape: [1]\ntemporal_blocking_interval: 5\n")
    assert c.length_per_node == [Fraction(1)]
    assert c.grid_per_node == [10] and c.grid_per_block == [10] and c.mpi_shape == [1]
    assert c.temporal_blocking_interval == 5
    assert c.filter_interval is None and c.with_omp is None


def test_3d_temporal_blocking_key_order_free():
    c = decode_config("length_per_node: [1.0,2.0,3.0]\nmpi_shape: [2,2,2]\ntemporal_blocking_interval: 5\n"
                      "grid_per_node: [10,10,10]\ngrid_per_block: [10,10,10]\nfilter_interval: 100\nwith_omp: 1\n")
    assert c.length_per_node == [1, 2, 3] and c.grid_per_node == [10, 10, 10]
    assert c.mpi_shape == [2, 2, 2] and c.grid_per_block == [10, 10, 10]
    assert c.temporal_blocking_interval == 5 and c.filter_interval == 100 and c.with_omp == 1


def test_3d_without_temporal_blocking():
    c = decode_config("length_per_node: [1.0,2.0,3.0]\nmpi_shape: [2,2,2]\ngrid_per_node: [10,10,10]\n")
    assert c.grid_per_block is None and c.temporal_blocking_interval is None
    assert c.filter_interval is None and c.with_omp is None


@pytest.mark.parametrize("text", [
    "length_per_node: [1.0]\ngrid_per_block: [10]\n",
    "length_per_node: [1.0]\ngrid_per_node: [10]\ngrid_per_block: []\nmpi_shape: []\ntemporal_blocking_interval: 5\n",
    "length_per_node: [1.0]\ngrid_per_node: [10]\ngrid_per_block: [10]\nmpi_shape: [1]\ntemporal_blocking_interval: -5\n",
    "length_per_node: [1.0]\ngrid_per_node: [10]\nwith_omp: 3\n",
    "length_per_node: [1.0]\ngrid_per_node: [10]\nfilter_interval: 0\n",
])
def test_invalid(text):
    with pytest.raises(ConfigError):
        decode_config(text)


def test_blocking_divisibility():
    # (N + 2*s*nt) must be a multiple of grid_per_block
    nc = decode_config("length_per_node: [1.0]\ngrid_per_node: [100]\ngrid_per_block: [10]\n"
                       "temporal_blocking_interval: 5\n")
    ic = convert_config(1, None, None, nc)
    assert ic.blocking.temporal and ic.blocking.block_per_node == [11] and ic.blocking.nt == 5
    assert convert_config(2, None, None, nc).blocking.block_per_node == [12]   # 100 + 2*2*5 = 120
    nc2 = decode_config("length_per_node: [1.0]\ngrid_per_node: [100]\ngrid_per_block: [7]\n"
                        "temporal_blocking_interval: 5\n")
    with pytest.raises(ConfigError):
        convert_config(1, None, None, nc2)


def test_filter_interval_multiple_of_nt():
    nc = decode_config("length_per_node: [1.0]\ngrid_per_node: [100]\ngrid_per_block: [10]\n"
                       "temporal_blocking_interval: 5\nfilter_interval: 7\n")
    with pytest.raises(ConfigError):
        convert_config(1, None, None, nc)


def test_space_interval_is_double_division():
    nc = decode_config("length_per_node: [40.96, 1.0]\ngrid_per_node: [4096, 3]\n")
    ic = convert_config(1, None, None, nc)
    assert ic.space_interval == [40.96 / 4096, 1.0 / 3]
