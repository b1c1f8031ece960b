"""The autotuner times the exposed kernel-shape variants on a real system and caches the winner."""
import json
import os

import numpy as np
import pytest

from systems import liquid

pytestmark = pytest.mark.gpu


def test_tune_system_picks_a_candidate_and_caches(cuda_lib, tmp_path, monkeypatch):
    from pis_gb300 import autotune
    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "tune.json"))
    s = liquid(nc=8, seed=3)
    opt = autotune.tune_system(s["table"], 1, s["pos"], s["types"], s["masses"], s["h"], s["vel"],
                               precision="mixed", steps=20, use_cache=False)
    assert opt in autotune.MIXED_CANDIDATES
    d = json.load(open(tmp_path / "tune.json"))
    (key, rec), = d.items()
    assert "|mixed|" in key and len(rec["all"]) == len(autotune.MIXED_CANDIDATES)
    assert rec["ms_per_step"] == min(a["ms_per_step"] for a in rec["all"])
    # second call is served from the cache
    assert autotune.tune_system(s["table"], 1, s["pos"], s["types"], s["masses"], s["h"], s["vel"],
                                precision="mixed") == opt
