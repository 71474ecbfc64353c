"""Host-side loop logic (no GPU): the nodal form of the volume averages and the field schedule."""

import numpy as np

from mumag_matrixfree2_gb300 import synthetic as syn
from mumag_matrixfree2_gb300.hysteresis_loop import NodalAverages, volume_averaged_J_parallel, volume_averaged_m

from .helpers import case, random_state


def test_nodal_averages_equal_the_element_form():
    """src/hysteresis_loop.py:153-223 averages over elements; the nodal weights give the same numbers."""
    s, p, _ = case("cube16_h2_air48")
    g = s.geom
    av = NodalAverages(g.conn, g.volume, g.mat_id, s.Js_lookup, s.N)
    for seed in (0, 1, 2):
        m = random_state(s.N, seed=seed)
        h = syn.tilted_field_direction(10.0 * seed + 1.0)
        J = volume_averaged_J_parallel(m, g.conn, g.volume, g.mat_id, s.Js_lookup, h)
        assert abs(av.J_parallel(m, h) - J) <= 1e-14 * max(1.0, abs(J))
        ma = volume_averaged_m(m, g.conn, g.volume, g.mat_id, s.Js_lookup)
        assert np.max(np.abs(av.m_avg(m) - ma)) <= 1e-14


def test_field_schedule_matches_the_reference_rule():
    """src/hysteresis_loop.py:128-150: floor(|span|/dB) + 1 values ending exactly at B_end; loop mirrors."""
    B = syn.field_values(8.0, -8.0, 0.1, False)
    assert len(B) == 161 and B[0] == 8.0 and B[-1] == -8.0
    B2 = syn.field_values(8.0, -8.0, 0.2, False)
    assert len(B2) == 81
    Bl = syn.field_values(1.0, -1.0, 0.5, True)
    assert np.allclose(Bl, [1.0, 0.5, 0.0, -0.5, -1.0, -0.5, 0.0, 0.5, 1.0])


def test_coercive_field_matches_the_oracle_evaluation():
    from mumag_matrixfree2_gb300.hysteresis_loop import coercive_field
    from oracle.minimize import compute_coercivity

    B = np.linspace(8.0, -8.0, 161)
    for shift in (-6.03, -0.55, 2.0):
        J = 1.6 * np.tanh(3.0 * (B - shift))
        assert coercive_field(B, J) == compute_coercivity(B, J)
    J = np.where(B > -6.0, 1.6, -1.6)  # a hard switch between two field values
    assert coercive_field(B, J) == compute_coercivity(B, J)
