"""The grid workloads built from arrays equal the same grids added to a
`CircuitBuilder` device by device: node numbering, device names, groups,
parameters and segments."""

import sys
from pathlib import Path

import pytest
import torch

from voltax_gb300 import workloads
from voltax_gb300.builder import CircuitBuilder

sys.path.insert(0, str(Path(__file__).parent))
from circuits import grid_via_builder  # noqa: E402


def assert_same_circuit(a, b):
    assert a.layout == b.layout
    assert a.node_segment == b.node_segment
    assert sorted(a.elements) == sorted(b.elements)
    for name in a.elements:
        x, y = a.elements[name], b.elements[name]
        assert type(x) is type(y) and x.nodes == y.nodes, name
        for f in x.fields:
            assert torch.equal(getattr(x, f), getattr(y, f)), (name, f)
        if hasattr(x, "value"):
            assert type(x.value) is type(y.value)
            for p, q in zip(x.value.params(), y.value.params()):
                assert torch.equal(p, q), name
            assert torch.equal(x.ac, y.ac) and torch.equal(x.ac_phase, y.ac_phase)
    assert a.topology_key() == b.topology_key()


@pytest.mark.parametrize("n,seed", [(2, 0), (3, 1), (10, 0), (26, 5), (60, 2)])
def test_power_grid_equals_builder(n, seed):
    assert_same_circuit(workloads.power_grid(n, seed), grid_via_builder(n, seed))


def test_power_grid_batch_equals_builder():
    sides = [7, 12, 4, 30]
    b = CircuitBuilder()
    for k, n in enumerate(sides):
        grid_via_builder(n, 3 + k, prefix=f"g{k}_", b=b)
    c = b.build()
    seg = [int(name[1:name.index("_")]) for name in c.layout.node_names]
    assert_same_circuit(workloads.power_grid_batch(sides, seed=3), c.with_segments(seg))
