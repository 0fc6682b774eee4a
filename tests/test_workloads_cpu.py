"""The benchmark workloads have the sizes the scope table states: global
elements per side n_g = N m + N - 1, global DOFs (n_g + 2p - 1)^2 and the
cell sides of the first, interior and last cells (m + 4, m + 6, m + 2
elements plus 2p - 1)."""
import pytest

from lsweeps.capi import geometry_cell
from lsweeps.problems import config

# (N, m, p, n_g, global DOFs, cell DOF sides {first, interior, last})
EXPECTED = {
    "C1": (4, 64, 10, 259, 77_284, {87, 89, 85}),
    "C2": (8, 128, 16, 1031, 1_127_844, {163, 165, 161}),
    "C3": (16, 128, 20, 2063, 4_418_404, {171, 173, 169}),
    "C4": (32, 128, 20, 4127, 17_355_556, {171, 173, 169}),
}


@pytest.mark.parametrize("name", sorted(EXPECTED))
def test_workload_sizes(name):
    N, m, p, n_g, dofs, sides = EXPECTED[name]
    spec, med = config(name)
    assert (spec.N, spec.m, spec.p) == (N, m, p)
    assert spec.n_g == n_g and spec.n_dof ** 2 == dofs
    assert med.shape == (spec.n_dof, spec.n_dof)
    # cell index I N + J: the x-lines follow J, the points per line follow I
    assert {geometry_cell(N, m, p, spec.h, j)["nx"] for j in (0, 1, N - 1)} == sides
    assert {geometry_cell(N, m, p, spec.h, i * N)["ny"] for i in (0, 1, N - 1)} == sides


def test_c3_has_64_sources_and_c4_one():
    assert len(config("C3")[0].sources) == 64
    assert len(config("C4")[0].sources) == 1
