"""The synthetic workloads are host-independent: the committed digests of small instances of every
family (tests/golden/synth_digests.json) must come out on every machine.  The CPU suite checks them
on the build host; the same check is marked gpu so that it also runs where the GPU suite runs (an
aarch64 host), which pins the x86-64 / aarch64 agreement."""
import json
from pathlib import Path

import pytest

from nav24_gb300.synth import Synth

CASES = json.loads((Path(__file__).resolve().parent / "golden" / "synth_digests.json").read_text())


def _check():
    for case in CASES:
        kw = {k: v for k, v in case.items() if k != "digest"}
        assert Synth(**kw).digest() == case["digest"], kw


def test_synth_digests():
    _check()


@pytest.mark.gpu
def test_synth_digests_on_the_gpu_host():
    _check()
