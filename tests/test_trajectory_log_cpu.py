"""The per-trajectory JSON-lines log of the study runner (the diagnostics of
HybridMonteCarloDiagnostic, src/simulation/monte_carlo/hybrid_monte_carlo.rs:402-410, kept for every
trajectory): one valid JSON object per trajectory with every field, appended."""
import json

import pytest


def test_trajectory_log_lines(tmp_path):
    import studies

    path = tmp_path / "run.jsonl"
    log = studies.TrajectoryLog(str(path))
    for k in range(3):
        log.write(trajectory=k, form="mixed", beta=2.0, delta_h=1e-7 * k, prob=1.0, accepted=1, plaquette=0.5,
                  gauss_steps=33, ms=13.5)
    log.close()
    log = studies.TrajectoryLog(str(path))
    log.write(trajectory=3, form="f64", beta=2.0, delta_h=-2e-7, prob=0.9, accepted=0, plaquette=0.5,
              gauss_steps=105, ms=555.0)
    with pytest.raises(ValueError):
        log.write(trajectory=4, form="f64")
    log.close()
    rows = [json.loads(line) for line in path.read_text().splitlines()]
    assert [r["trajectory"] for r in rows] == [0, 1, 2, 3]
    assert all(set(r) == set(studies.TrajectoryLog.KEYS) for r in rows)
    assert rows[3]["accepted"] is False and rows[0]["accepted"] is True
    studies.TrajectoryLog(None).write(trajectory=0)  # no path: nothing is written or checked
