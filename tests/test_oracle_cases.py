"""The oracle's own restatement of the timed workloads' initial conditions
(used by bench.py's CPU baseline and reference arm, which load nothing of
the library) agrees bit for bit with the library's host set-up
(gfm_case_params / gfm_case_init / gfm_case_shock_bubble)."""
import numpy as np
import pytest

import gfm_gb300 as g
import oracle_binding as orc

DESC_FIELDS = [f for f, _ in g.GridDesc._fields_]


@pytest.mark.parametrize("sim,case,Nx,Ny", [("onefluid", "circularexplosion", 200, 200),
                                            ("twofluid", "shock_bubble", 1000, 400),
                                            ("twofluid", "underwater_explosion_sg", 120, 120),
                                            ("twofluid", "shock_bubble", 96, 40)])
def test_workload_initial_conditions(sim, case, Nx, Ny):
    d, T, U1, U2, phi = orc.case_setup(sim, case, Nx, Ny)
    dg, Tg = g.case_params(sim, case, Nx, Ny)
    V1, V2, vphi = g.case_init(sim, case, dg)
    assert [getattr(d, f) for f in DESC_FIELDS] == [getattr(dg, f) for f in DESC_FIELDS] and T == Tg
    assert np.array_equal(U1, V1)
    if sim == "twofluid":
        assert np.array_equal(U2, V2) and np.array_equal(phi, vphi)


@pytest.mark.parametrize("member", [(128, 128, 1.1, 1.09, 0.1, 0.1), (1024, 384, 3.0, 1.67, 10.0, 0.3),
                                    (576, 256, 1.7, 1.3, 0.7, 0.22)])
def test_batch_family_initial_conditions(member):
    d, T, U1, U2, phi = orc.bubble_setup(*member)
    dg, Tg, V1, V2, vphi = g.shock_bubble_case(*member)
    assert [getattr(d, f) for f in DESC_FIELDS] == [getattr(dg, f) for f in DESC_FIELDS] and T == Tg
    assert np.array_equal(U1, V1) and np.array_equal(U2, V2) and np.array_equal(phi, vphi)
