"""Power sampling (gu_power_*) against a fake NVML library on the host: the
sampler reads only, so no GPU is needed to check its averaging and errors."""
import os
import subprocess
import time

import pytest

import gu
from conftest import ROOT


@pytest.fixture(scope="module")
def fake_nvml(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("nvml") / "libfake_nvml.so")
    r = subprocess.run(["gcc", "-shared", "-fPIC", "-O2", os.path.join(ROOT, "tests", "cpp", "fake_nvml.c"),
                        "-o", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_mean_power_and_samples(fake_nvml, monkeypatch):
    monkeypatch.setenv("GU_NVML_LIBRARY", fake_nvml)
    with gu.PowerSampler(device=0, period_ms=1) as p:
        time.sleep(0.05)
    assert abs(p.watts - 123.456) < 1e-9
    assert p.samples >= 2


def test_failing_reads_and_missing_library(fake_nvml, monkeypatch, tmp_path):
    monkeypatch.setenv("GU_NVML_LIBRARY", fake_nvml)
    monkeypatch.setenv("FAKE_NVML_FAIL", "1")
    with pytest.raises(gu.GuError) as e:
        with gu.PowerSampler(0, 1):
            time.sleep(0.01)
    assert e.value.status == 7
    monkeypatch.delenv("FAKE_NVML_FAIL")
    with pytest.raises(gu.GuError) as e:  # no such NVML device
        with gu.PowerSampler(3, 1):
            pass
    assert e.value.status == 1
    monkeypatch.setenv("GU_NVML_LIBRARY", str(tmp_path / "no_such_nvml.so"))
    with pytest.raises(gu.GuError) as e:
        with gu.PowerSampler(0, 1):
            pass
    assert e.value.status == 7
