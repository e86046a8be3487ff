r"""bench.py's `config` object: both arms build it from the same function of
the workload's sizes, so the GPU line and the reference line carry the same
keys and values; its L2 note names what a step streams (the FP32 values of
the implicit-column FullCI form, nothing per entry for the implicit DOCI form)
and the eigensolver's FP32 subspace."""

import pytest

import bench


@pytest.fixture(autouse=True)
def keep_workload():
    saved = bench.WORKLOAD
    yield
    bench.WORKLOAD = saved


def config(name, ndet, size, world=1):
    bench.WORKLOAD = bench.WORKLOADS[name]
    return bench.workload_config(ndet, 2 * size - ndet, size, world)


def test_config_keys_and_values():
    c = config("fci12", 627264, 538506144)
    assert set(c) == {"workload", "ndet", "nnz_stored", "nnz_reference", "roots", "tol", "l2", "parallelism"}
    assert c["ndet"] == 627264 and c["nnz_stored"] == 1076385024 and c["nnz_reference"] == 538506144
    assert c["roots"] == 4 and c["parallelism"] == "single GPU"
    # The same inputs give the same object (the two arms compare equal).
    assert c == config("fci12", 627264, 538506144)
    assert config("fci12", 627264, 538506144, world=2)["parallelism"] == "replicas"


def test_l2_note():
    fci = config("fci12", 627264, 538506144)["l2"]
    assert fci.startswith("4.31 GB of FP32 values per product") and "no flush needed" in fci
    doci = config("doci32", 10518300, 1020275100)["l2"]
    assert doci.startswith("no per-entry bytes (implicit DOCI form)")
    assert "subspace 5.39 GB" in doci and "no flush needed" in doci
    small = config("doci24", 134596, 7402780)["l2"]
    assert "fits in the 129 MB L2" in small
