"""The dispatcher configuration files (no GPU needed: parsing and dispatch rules).

Flag4j reads ./configs/ReDeMatMult.properties, CmDeMatMult.properties and
GeneralConfigs.properties with java.util.Properties and Integer.parseInt /
Double.parseDouble (src/main/java/org/flag4j/linalg/ops/dispatch/configs/
ReDeMatMultDispatchConfigs.java:89-121, Cm128DeMatMultDispatchConfigs.java:85-108,
src/main/java/org/flag4j/concurrency/Configurations.java:68-88); the kernel it
then runs for a shape follows ReDeMatMultDispatcher.getFunc
(src/main/java/org/flag4j/linalg/ops/dispatch/ReDeMatMultDispatcher.java:184-237)
and Cm128DeMatMultDispatcher.getFunc (Cm128DeMatMultDispatcher.java:184-226).
"""
import os

import pytest


@pytest.fixture()
def cfg(lib):
    from flag4j_gb300 import configs
    configs.reset()
    yield configs
    configs.reset()


def write(tmp_path, name, text):
    d = tmp_path / "configs"
    d.mkdir(exist_ok=True)
    (d / name).write_text(text)
    return d


def test_defaults_are_the_reference_defaults(cfg):
    r = cfg.get(False)
    assert (r["small_threshold"], r["aspect_threshold"], r["square_mt_standard_threshold"],
            r["square_mt_reordered_threshold"], r["wide_mt_reordered_threshold"],
            r["square_sequential_vec_threshold"], r["min_dim_small_threshold"], r["cache_size"]) == \
        (2450, 2.0, 50, 2048, 25, 256, 10, 64.0)
    z = cfg.get(True)
    assert (z["small_threshold"], z["square_mt_standard_threshold"], z["square_mt_reordered_threshold"]) == \
        (512, 60, 2048)
    assert r["gpu_gemm_mode"] == "auto" and r["loaded"] == 0
    assert cfg.general()[0] == 64


def test_properties_syntax(cfg, tmp_path):
    d = write(tmp_path, "ReDeMatMult.properties",
              "# comment line\n"
              "! another comment\n"
              "\n"
              "   smallThreshold = 100\n"
              "aspectThreshold: 3.5d\n"
              "squareMtStandardThreshold 70\n"
              "squareMtReorderedThreshold = 40\\\n"
              "    96\n"
              "squareStandardVecThreshold = 7\n"          # not a key the reference reads
              "squareSequentialVecThreshold=\\u0031\\u0032\n"  # unicode escapes: "12"
              "minDimSmallThreshold = 3\n"
              "minDimSmallThreshold = 4\n"                # the last one wins
              "unknownKey = whatever\n")
    cfg.load(d)
    r = cfg.get(False)
    assert r["loaded"] == 1
    assert r["small_threshold"] == 100
    assert r["aspect_threshold"] == 3.5
    assert r["square_mt_standard_threshold"] == 70
    assert r["square_mt_reordered_threshold"] == 4096
    assert r["square_sequential_vec_threshold"] == 12
    assert r["min_dim_small_threshold"] == 4
    assert r["wide_mt_reordered_threshold"] == 25  # absent: default
    assert cfg.get(True)["loaded"] == 0            # no CmDeMatMult.properties: complex defaults
    assert cfg.get(True)["small_threshold"] == 512


def test_number_syntax_errors_keep_the_previous_configuration(cfg, tmp_path):
    from flag4j_gb300 import _lib
    from flag4j_gb300.device import IllegalArgumentException
    good = write(tmp_path, "ReDeMatMult.properties", "smallThreshold = 777\n")
    cfg.load(good)
    bad = tmp_path / "bad"
    bad.mkdir()
    # Properties keeps trailing blanks in a value, and Integer.parseInt rejects them
    (bad / "ReDeMatMult.properties").write_text("smallThreshold = 2450  \n")
    with pytest.raises(IllegalArgumentException) as e:
        cfg.load(bad)
    assert 'NumberFormatException: For input string: "2450  "' in str(e.value)
    assert cfg.get(False)["small_threshold"] == 777
    (bad / "ReDeMatMult.properties").write_text("aspectThreshold = 2.0.1\n")
    with pytest.raises(IllegalArgumentException):
        cfg.load(bad)
    (bad / "ReDeMatMult.properties").write_text("smallThreshold = 2147483648\n")  # beyond int
    with pytest.raises(IllegalArgumentException):
        cfg.load(bad)
    (bad / "ReDeMatMult.properties").write_text("gpuGemmMode = fastest\n")
    with pytest.raises(IllegalArgumentException):
        cfg.load(bad)
    # Double.parseDouble trims blanks
    (bad / "ReDeMatMult.properties").write_text("aspectThreshold = 1.5   \n")
    cfg.load(bad)
    assert cfg.get(False)["aspect_threshold"] == 1.5
    assert _lib.load().f4j_config_get(0, None) == _lib.F4J_ERR_ARG


def test_general_configs_and_parallelism(cfg, tmp_path):
    nproc = os.cpu_count()
    for value, want in ((4, 4), (0, nproc), (-1, max(nproc - 1, 1)), (-100000, 1)):
        d = write(tmp_path, "GeneralConfigs.properties", "blockSize = 32\nparallelism = %d\n" % value)
        cfg.load(d)
        bs, par = cfg.general()
        assert bs == 32
        assert par == want, (value, par)


def test_gpu_gemm_mode_precedence(cfg, tmp_path):
    d = write(tmp_path, "GeneralConfigs.properties", "gpuGemmMode = plain\n")
    cfg.load(d)
    assert cfg.get(False)["gpu_gemm_mode"] == "plain" and cfg.get(True)["gpu_gemm_mode"] == "plain"
    write(tmp_path, "CmDeMatMult.properties", "gpuGemmMode = EXACT\n")
    cfg.load(d)
    assert cfg.get(False)["gpu_gemm_mode"] == "plain" and cfg.get(True)["gpu_gemm_mode"] == "exact"
    assert cfg.dispatch(1024, 1024, 1024)[0] == "plain"
    assert cfg.dispatch(1024, 1024, 1024, complex=True)[0] == "exact"


def test_auto_resolution_rules(cfg, tmp_path):
    # dataLength(A) + dataLength(B) < smallThreshold -> the reference's order
    assert cfg.dispatch(24, 24, 24)[0] == "exact"            # 1152 entries
    # at most 2^24 flops -> the reference's order as well
    assert cfg.dispatch(200, 200, 200)[0] == "exact"
    assert cfg.dispatch(300, 300, 300)[0] == "split"
    assert cfg.dispatch(300, 300, 300, mode="plain")[0] == "plain"   # explicit modes are kept
    d = write(tmp_path, "ReDeMatMult.properties", "smallThreshold = 200000\n")
    cfg.load(d)
    assert cfg.dispatch(300, 300, 300)[0] == "exact"         # 180000 entries < 200000
    assert cfg.dispatch(300, 300, 400)[0] == "split"         # 240000 entries
    assert cfg.dispatch(300, 300, 300, complex=True)[0] == "split"  # CmDeMatMult defaults


def test_reference_kernel_choice(cfg):
    # (m, n, k) of C = A (m x k) B (k x n) -> the kernel ReDeMatMultDispatcher.getFunc picks
    real = {
        (10, 10, 10): "STRD",               # 200 entries: dispatch()'s small path
        (1024, 1024, 1024): "MT_REORD",     # near square, inner 1024 < 2048
        (8192, 8192, 8192): "MT_BLK_REORD",
        (64, 64, 40): "MT_STRD",            # near square, inner 40 < 50
        (4096, 4096, 2048): "MT_BLK_REORD",  # aspect 2.0 <= 2.0, inner 2048
        (4096, 64, 8): "STRD",              # m the largest, smallest dim 8 < 10
        (4096, 64, 64): "MT_REORD",
        # getFunc's n is the inner dimension and its k the columns of C
        (20, 64, 4096): "MT_STRD",          # inner the largest, m 20 < 25
        (64, 64, 4096): "MT_REORD",
        (4, 64, 4096): "STRD",              # inner the largest, smallest dim 4 < 10
        (64, 4096, 64): "MT_REORD",         # columns of C the largest
        (64, 4096, 4): "REORD",
        (20, 4096, 64): "MT_REORD",
        (300, 1, 300): "MT_BLK_VEC_AS_MAT",  # matrix-vector, near square, m >= 256
        (200, 1, 200): "BLK_VEC_AS_MAT",
        (4000, 1, 100): "BLK_VEC_AS_MAT",   # aspect 40 > 8
    }
    for (m, n, k), want in real.items():
        assert cfg.dispatch(m, n, k)[1] == want, ((m, n, k), cfg.dispatch(m, n, k))
    assert cfg.dispatch(300, 1, 300, complex=True)[1] == "MT_STRD_VEC_AS_MAT"
    assert cfg.dispatch(64, 64, 55, complex=True)[1] == "MT_STRD"  # complex: inner 55 < 60


def test_reads_dot_configs_of_the_working_directory(cfg, tmp_path, monkeypatch):
    write(tmp_path, "ReDeMatMult.properties", "smallThreshold = 31337\n")
    monkeypatch.chdir(tmp_path)
    cfg.load()
    assert cfg.get(False)["small_threshold"] == 31337
