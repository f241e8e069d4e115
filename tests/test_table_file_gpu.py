"""Table files loaded into device memory and joined: the reference's own
join_ori known answer through the raw format, and device round trips through
both formats."""
import numpy as np
import pytest
import torch

from eating_one_gb300 import native
from eating_one_gb300.engine import JoinError
from oracle import oracle as O
from tests import golden

pytestmark = pytest.mark.gpu


def test_join_ori_from_files(engine, tmp_path):
    R, S = golden.join_ori()
    R.tofile(tmp_path / "R")
    S.tofile(tmp_path / "S")
    dR = engine.load_table(str(tmp_path / "R"), native.EJ_TABLE_FILE_RAW)
    dS = engine.load_table(str(tmp_path / "S"), native.EJ_TABLE_FILE_RAW)
    assert torch.equal(dR.cpu(), torch.from_numpy(R)) and torch.equal(dS.cpu(), torch.from_numpy(S))
    runs = golden.reference_runs()["join_ori"]
    for algo in ("hash", "bnl", "hash_index", "sort_index"):
        rows = engine.join(algo, dR, dS).cpu().numpy()
        assert rows.shape[0] == 1002230
        # the value every reference join_ori program prints (resultVal = sum of rval)
        assert set(runs.values()) == {int(rows[:, 1].astype(np.int64).sum())}
        assert np.array_equal(O.canon(rows), O.canon(O.hash_join(R, S)))


@pytest.mark.parametrize("n", [0, 1, 4_000_001])
def test_device_round_trip(engine, tmp_path, n):
    rng = np.random.default_rng(n)
    rows = torch.from_numpy(rng.integers(-2 ** 31, 2 ** 31, size=(n, 2), dtype=np.int64).astype(np.int32))
    dev = rows.cuda()
    for fmt, name in ((native.EJ_TABLE_FILE_COUNTED, "t.tbl"), (native.EJ_TABLE_FILE_RAW, "t.raw")):
        engine.save_table(str(tmp_path / name), dev, fmt)  # from device memory (chunked copies)
        assert np.array_equal(native.read_table_file(str(tmp_path / name), fmt), rows.numpy())
        back = engine.load_table(str(tmp_path / name), fmt)
        assert torch.equal(back.cpu(), rows)
    engine.save_table(str(tmp_path / "h.tbl"), rows)  # from host memory
    assert torch.equal(engine.load_table(str(tmp_path / "h.tbl")).cpu(), rows)


def test_load_errors(engine, tmp_path):
    with pytest.raises(JoinError, match="EJ_ERR_IO|cannot read"):
        engine.load_table(str(tmp_path / "missing.tbl"))
    rows = torch.arange(20, dtype=torch.int32).reshape(10, 2).cuda()
    engine.save_table(str(tmp_path / "t.tbl"), rows)
    import ctypes as C

    small = torch.empty((4, 2), dtype=torch.int32, device="cuda")
    n = C.c_uint64(0)
    st = engine.lib.ej_table_load(engine.h, str(tmp_path / "t.tbl").encode(), native.EJ_TABLE_FILE_COUNTED,
                                  C.c_void_p(small.data_ptr()), 4, C.byref(n))
    assert st == native.EJ_ERR_CAPACITY and n.value == 10


@pytest.mark.parametrize("algo", ["hash", "sort_index"])
def test_cli_on_join_ori_files(tmp_path, algo):
    """The command-line driver (mirroring the reference executables) on the
    join_ori files: the reference's match count, for the host and device paths."""
    import subprocess

    from eating_one_gb300.build import CLI_PATH

    R, S = golden.join_ori()
    R.tofile(tmp_path / "R")
    S.tofile(tmp_path / "S")
    for extra in ([], ["--host"]):
        out = subprocess.run([CLI_PATH, algo, "0", "0", "--raw", str(tmp_path / "R"), str(tmp_path / "S")] + extra,
                             check=True, capture_output=True, text=True, timeout=120).stdout
        assert "the number of total match tuple = 1002230" in out
