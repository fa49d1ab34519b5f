"""What the trained bit selector gains over the rule on fresh systems (not in
the training sweep), solved by the batched engine on the GPU: the selected F
is computed by the library's MLP kernels from the matrix features."""
import numpy as np
import pytest

import bitsel
import sagb

pytestmark = pytest.mark.gpu

# anisotropic 2D systems (where the rule's F overflows the int32 range) and 3D
# Poisson / convection-diffusion, with seeds outside the training set
CASES = [(sagb.GEN_ANISO2D, 300, 3e-4, 9001), (sagb.GEN_ANISO2D, 250, 2e-3, 9002),
         (sagb.GEN_POISSON3D, 36, 0.0, 9003), (sagb.GEN_CONVDIFF3D, 32, 40.0, 9004),
         (sagb.GEN_STENCIL27, 30, 0.0, 9005)]


@pytest.fixture(scope="module")
def ctx():
    c = sagb.Context(0)
    yield c
    c.close()


def test_selector_beats_rule(ctx):
    sel = bitsel.Selector(ctx)
    tot_sel = tot_rule = 0
    rule_failed = 0
    for spec in CASES:
        r, c, v, b = bitsel.make_system(spec)
        B = sagb.Batch(ctx, [(r, c, v)] * 2, 1)
        nrm = float(np.linalg.norm(b))
        q = float(B.rule_ratios(np.concatenate([b, b]), [nrm, nrm])[0])
        rule = bitsel.rule_of(q)
        f = sel.choose(sagb.setup_features(B.system_setup(0), q), rule)
        x = np.zeros(B.rows)
        p = sagb.solver_params(m=30, max_outer=4, explicit_stop=1, overflow_fallback=0)
        it, cv, fb = B.solve(p, [f, rule], np.concatenate([b, b]), [nrm, nrm], x)
        assert cv[0] == 1, (spec, f, it)          # the selected F converges
        tot_sel += int(it[0])
        tot_rule += int(it[1]) if cv[1] else 120  # a failed rule F costs the sweep's cap
        rule_failed += int(not cv[1])
        B.close()
    print("selected / rule iterations:", tot_sel, tot_rule, "rule failures:", rule_failed)
    assert tot_sel < tot_rule
    sel.net.close()
