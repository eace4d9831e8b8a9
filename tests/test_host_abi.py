"""CPU-side checks of the product library: it loads, exports every symbol the
public header declares, and its C++ reader/preprocessing (the drop-in
MESHBLOCK/SOLNBLOCK) is bit-identical to the oracle's.  No GPU calls."""
import numpy as np
import pytest


def test_library_exports_header_symbols(native_lib):
    from hamstr_oop_gb300 import native
    declared = native.declared_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if not hasattr(native_lib, s)]
    assert not missing, missing


def test_shape_keys_match_the_header():
    """The Python shape keys and the header's HAMSTR_SHAPE_N (the length of
    the array hamstr_gpu_get_shape / set_shape read and write) agree, and the
    header documents every index."""
    import os
    import re
    from hamstr_oop_gb300 import native
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "hamstr_gpu.h")
    text = open(hdr).read()
    n = int(re.search(r"#define HAMSTR_SHAPE_N (\d+)", text).group(1))
    assert n == len(native.GpuSolver.SHAPE_KEYS) == len(set(native.GpuSolver.SHAPE_KEYS))
    for i in range(n):
        assert re.search(r"\*\s+\[%d\] " % i, text), i


@pytest.mark.parametrize("ni,nj,order,loop_start", [(16, 4, 3, None), (24, 6, 5, 0), (40, 8, 1, 3)])
def test_reader_and_preprocess_match_oracle(make_case, oracle_lib, native_lib, ni, nj, order, loop_start):
    from hamstr_oop_gb300 import native
    case = make_case(ni, nj, order=order, loop_start=loop_start)
    host = native.Case(case)
    orc = oracle_lib.OracleCase(case, "port")
    assert host.sizes == orc.sizes
    assert host.params == orc.params
    for name in ("faces", "chainConn", "faceStartPerChain", "c2chain", "bFaces", "chainsPerColor"):
        assert np.array_equal(host.get_int(name), orc.get_int(name)), name
    for name in ("x", "vol", "normVec", "refMtx", "q"):
        assert np.array_equal(host.get(name), orc.get(name)), name


def test_missing_case_is_an_error_not_an_exit(tmp_path, native_lib):
    from hamstr_oop_gb300 import native
    with pytest.raises(native.HamstrError) as ei:
        native.Case(str(tmp_path / "nothing"))
    assert ei.value.status == -5


def test_truncated_mesh_file_is_an_error(make_case, native_lib):
    import os
    from hamstr_oop_gb300 import native
    case = make_case(16, 4)
    p = os.path.join(case, "input", "domain000", "qedges.dat")
    lines = open(p).read().splitlines()
    open(p, "w").write("\n".join(lines[: len(lines) // 2]) + "\n")
    with pytest.raises(native.HamstrError) as ei:
        native.Case(case)
    assert ei.value.status == -5


def test_testcase_nonzero_rejected(make_case, native_lib):
    from hamstr_oop_gb300 import native
    case = make_case(16, 4, testcase=1)
    with pytest.raises(native.HamstrError):
        native.Case(case)


def test_every_status_code_has_a_message(native_lib):
    """Each HAMSTR_GPU_ERR_* of the header has its own hamstr_gpu_strerror text."""
    import os
    import re
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "hamstr_gpu.h")
    codes = [int(v) for v in re.findall(r"#define HAMSTR_GPU_ERR_\w+\s+(-\d+)", open(hdr).read())]
    assert len(codes) >= 8 and len(set(codes)) == len(codes)
    msgs = [native_lib.hamstr_gpu_strerror(c).decode() for c in codes]
    assert "unknown status" not in msgs and len(set(msgs)) == len(msgs)
