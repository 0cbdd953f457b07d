"""The autotuner's cache (voxelfem_gb300.autotune) on the host: keys name the grid shape, the
coarsening count, the precision, the initial-guess method and the GPU, and lookups read back what
a tuning run wrote."""
import json

from voxelfem_gb300 import autotune


class _Sim:
    NbElementsPerDimension = [128, 128, 128]


class _Solver:
    numLevels = 6
    _prec = "mixed"


def test_key_and_lookup(tmp_path):
    k = autotune.key(_Sim(), _Solver(), "zero", device="NVIDIA GB300")
    assert k == "lbl|128x128x128|c5|mixed|zero|NVIDIA GB300"
    path = tmp_path / "cache.json"
    entry = {"slots": 8, "sweepForm": "lines", "mgSmoothingIterations": 2, "seconds": 0.1}
    path.write_text(json.dumps({k: entry}))
    data = autotune.load(str(path))
    assert data[k]["sweepForm"] == "lines"
    assert autotune.load(str(tmp_path / "missing.json")) == {}


def test_shipped_cache_is_well_formed():
    data = autotune.load()
    for k, e in data.items():
        assert k.startswith("lbl|")
        assert e["sweepForm"] in ("lines", "colours", "planes", "staged")
        assert e["slots"] >= 1 and e["mgSmoothingIterations"] >= 1
