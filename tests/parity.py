"""Comparison helpers shared by the oracle (CPU) and GPU parity tests."""
import numpy as np

# FP64 plain path: every amplitude within this of the reference, scaled by
# the largest amplitude magnitude of the case (debug states are unnormalised).
AMP_TOL = 1e-12
PROBE_TOL = 1e-11


def check_case(case, amps, results, probes, ref_amps):
    scale = max(1.0, float(np.max(np.abs(ref_amps))) if ref_amps.size else 1.0)
    err = float(np.max(np.abs(amps - ref_amps))) if ref_amps.size else 0.0
    assert err <= AMP_TOL * scale, f"{case['name']}: max |d amp| = {err:.3e}"
    assert len(results) == len(case["results"]), case["name"]
    for got, want in zip(results, case["results"]):
        if isinstance(want, int):
            assert got == want, f"{case['name']}: outcome {got} != {want}"
        else:
            assert abs(got - want) <= PROBE_TOL * max(1.0, abs(want)), f"{case['name']}: {got} != {want}"
    for p, got, want in zip(case["probes"], probes, case["probe_values"]):
        got, want = np.asarray(got), np.asarray(want)
        tol = PROBE_TOL * max(1.0, float(np.max(np.abs(want))))
        assert got.shape == want.shape and np.max(np.abs(got - want)) <= tol, \
            f"{case['name']} probe {p[0]}: {got} vs {want}"
