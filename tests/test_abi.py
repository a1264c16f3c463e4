"""The C ABI: the shared library loads and exports every function include/*.h declares,
and the ctypes signature table matches the header (CPU only, no compute calls)."""
import re
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"RL_API[^;{]*?\b(rl_\w+)\s*\(", text, flags=re.S))
    return names


def test_header_declares_entry_points():
    names = declared()
    assert {"rl_dgemm", "rl_dlu_decompose", "rl_dcholesky_solve", "rl_dqr_decompose",
            "rl_dbatch_solve_dev"} <= names


def test_library_exports_every_declared_symbol(rl):
    out = subprocess.run(["nm", "-D", "--defined-only", str(rl.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\b(rl_\w+)$", out, flags=re.M))
    missing = declared() - exported
    assert not missing, missing
    for name in declared():
        assert hasattr(rl.lib, name)


def test_signature_table_matches_header(rl):
    from rulinalg_gb300._lib import SIGNATURES
    assert set(SIGNATURES) == declared()


def test_status_strings_and_device_check(rl):
    assert rl.lib.rl_status_string(0) == b"ok"
    assert b"division by zero" in rl.lib.rl_status_string(4)
    assert rl.lib.rl_version() >= 100
    st = rl.lib.rl_device_check()
    assert st in (0, 33)  # 33 = RL_ERR_NO_DEVICE on a machine without an sm_103 GPU


def test_no_device_fails_loudly(rl):
    """Without a GPU every compute entry point returns RL_ERR_NO_DEVICE (no CPU path)."""
    import numpy as np
    import pytest
    if rl.device_available():
        pytest.skip("a GPU is present")
    a = np.eye(3)
    with pytest.raises(rl.DeviceError):
        rl.mat_mul(a, a)
    with pytest.raises(rl.DeviceError):
        rl.PartialPivLu.decompose(a)


def test_tunables_ranges_and_defaults(rl):
    """rl_tune_set / rl_tune_get need no GPU: defaults, range checks, unknown keys."""
    from rulinalg_gb300 import _lib as L
    defaults = {L.TUNE_WAIT_TIMEOUT_NS: 10 ** 9, L.TUNE_PANEL_CLUSTER_MAX: 16, L.TUNE_BATCH_CTAS_PER_SM: 0,
                L.TUNE_BATCH_WARP_COST: 32768, L.TUNE_UPLOAD_CHUNKS: 32, L.TUNE_MIXED_REFINE_STEPS: 30,
                L.TUNE_LU_OUTER_NB: -1, L.TUNE_MIXED_SWEEP_INV: 1, L.TUNE_PANEL_LOOKAHEAD: 0, L.TUNE_FULLPIV_CTAS_PER_SM: 3, L.TUNE_TEST_WITHHOLD_CHUNK: -1,
                L.TUNE_TEST_WITHHOLD_SWEEP_BLOCK: -1}
    for k, v in defaults.items():
        assert rl.tune_get(k) == v
    import pytest
    for k, bad in ((L.TUNE_WAIT_TIMEOUT_NS, 0), (L.TUNE_PANEL_CLUSTER_MAX, 17), (L.TUNE_UPLOAD_CHUNKS, 0),
                   (L.TUNE_BATCH_WARP_COST, 40000), (L.TUNE_TEST_WITHHOLD_CHUNK, -2), (L.TUNE_LU_OUTER_NB, 4097),
                   (L.TUNE_LU_OUTER_NB, -2), (L.TUNE_MIXED_SWEEP_INV, 2), (999, 1)):
        with pytest.raises(ValueError):
            rl.tune_set(k, bad)
    rl.tune_set(L.TUNE_UPLOAD_CHUNKS, 7)
    assert rl.tune_get(L.TUNE_UPLOAD_CHUNKS) == 7
    rl.tune_set(L.TUNE_UPLOAD_CHUNKS, 32)
    for k, v in defaults.items():
        assert rl.tune_get(k) == v
