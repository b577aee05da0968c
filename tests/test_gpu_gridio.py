"""Grid results I/O: the `;`-separated text dump of the reference's examples
(msl_grid_dump_text) byte-for-byte against the oracle's std::ofstream
restatement, and the reader (msl_grid_load_text) on its output.
"""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

SPECIAL = [0.0, -0.0, np.nan, np.inf, -np.inf, 1e-40, -3.0e38, 1e-5, 123456.7, 1234567.0, 0.1, 2.0 / 3.0]


def grid(shape, dtype, seed):
    g = np.random.default_rng(seed)
    if dtype == np.int32:
        return g.integers(-2**31, 2**31, shape, dtype=np.int64).astype(np.int32)
    x = (g.standard_normal(shape) * 10.0 ** g.integers(-8, 8, shape)).astype(dtype)
    flat = x.reshape(-1)
    flat[:len(SPECIAL)] = np.array(SPECIAL[:flat.size], dtype)
    return x


@pytest.mark.parametrize("shape", [(1, 1), (3, 5), (64, 70), (2, 3, 4), (5, 17, 9), (33, 8, 40)],
                         ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.uint16])
def test_dump_matches_oracle_bytes(gpu, tmp_path, shape, dtype):
    x = grid(shape, dtype if dtype != np.uint16 else np.float32, sum(shape))
    if dtype == np.uint16:
        x = O.to_bf16(x)
    d = gpu.DeviceArray.from_host(x)
    mine, ref = tmp_path / "gpu.out", tmp_path / "oracle.out"
    gpu.grid_dump_text(str(mine), d)
    gpu.grid_dump_text(str(mine), d)  # appends, as the examples do
    O.dump_text(str(ref), x)
    O.dump_text(str(ref), x)
    assert mine.read_bytes() == ref.read_bytes()


@pytest.mark.parametrize("shape", [(7, 9), (4, 6, 5)], ids=lambda s: "x".join(map(str, s)))
def test_load_reads_the_dump(gpu, tmp_path, shape):
    xi = grid(shape, np.int32, 3)
    p = tmp_path / "i.out"
    O.dump_text(str(p), xi)
    back = gpu.DeviceArray(shape, np.int32)
    gpu.grid_load_text(str(p), back)
    assert np.array_equal(back.download(), xi)  # integers round-trip exactly
    xf = grid(shape, np.float32, 4)
    p = tmp_path / "f.out"
    O.dump_text(str(p), xf)
    back = gpu.DeviceArray(shape, np.float32)
    gpu.grid_load_text(str(p), back)
    # The text keeps 6 significant digits: the value read is the float nearest
    # to the printed decimal.
    want = np.array([np.float32(float("%g" % v)) for v in xf.ravel()], np.float32).reshape(shape)
    assert np.array_equal(back.download().view(np.uint32), want.view(np.uint32))


def test_load_rejects_bad_files(gpu, tmp_path):
    p = tmp_path / "short.out"
    p.write_text("1;2;3;\n4;5;\n")
    d = gpu.DeviceArray((2, 3), np.float32)
    with pytest.raises(gpu.MslError) as e:
        gpu.grid_load_text(str(p), d)
    assert e.value.code == gpu.MSL_ERR_SIZE_MISMATCH
    p.write_text("1;2;x;\n4;5;6;\n")
    with pytest.raises(gpu.MslError) as e:
        gpu.grid_load_text(str(p), d)
    assert e.value.code == gpu.MSL_ERR_INVALID_ARGUMENT
    p.write_text("1;2;3;\n4;5;6;7;\n")
    with pytest.raises(gpu.MslError) as e:
        gpu.grid_load_text(str(p), d)
    assert e.value.code == gpu.MSL_ERR_SIZE_MISMATCH
    with pytest.raises(gpu.MslError):
        gpu.grid_load_text(str(tmp_path / "missing.out"), d)


def test_heat2d_result_dump(gpu, tmp_path):
    """The heat2D example's output file for a 1024 x 1024 grid after 20 sweeps."""
    from muesli4_gb300 import workloads as W
    g = W.jacobi_grid(1024, 1024, seed=5)
    a, b = gpu.DeviceArray.from_host(g), gpu.DeviceArray(g.shape, np.float32)
    out = gpu.stencil2d_iterate(gpu.MSL_ST2_HEAT5, a, b, 1, 0.0, 20, residual=False)[0]
    mine, ref = tmp_path / "d2.out", tmp_path / "ref.out"
    gpu.grid_dump_text(str(mine), out)
    O.dump_text(str(ref), O.stencil2d_iterate(1, g, 1, 0.0, 20)[0])
    assert mine.read_bytes() == ref.read_bytes()
