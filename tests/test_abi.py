"""The C-ABI library loads and exports every entry point include/*.h declares.

Runs without a GPU: only symbol lookup, status strings and argument checks
that return before any device work.
"""
import ctypes as C
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(ttg_\w+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("ttg_round", "ttg_round_batch", "ttg_matvec_round", "ttg_matmat_round",
                 "ttg_eval_batch", "ttg_inner", "ttg_norm", "ttg_free",
                 "ttg_right_orthogonalize"):
        assert must in names


def test_library_exports_every_declared_symbol(ttg):
    lib = C.CDLL(ttg.library_path())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings_and_free(ttg):
    L = ttg.lib()
    assert L.ttg_status_string(0) == b"ok"
    assert L.ttg_status_string(4) == b"index out of range"
    t = ttg._Tensor()
    L.ttg_free(C.byref(t))  # not owned: no-op


def test_rejects_streaming_method_for_round(ttg):
    # round_assert_method_for_value (round/round.hpp:124-134) -- checked
    # before any device work, so this runs on a CPU-only host too.
    with pytest.raises(ttg.TTGError) as e:
        ttg.round([__import__("numpy").ones((1, 2, 1))],
                  ttg.RoundOptions(method=ttg.round_method.svd_streaming))
    assert e.value.status == 3


def test_rejects_unknown_schedule_and_precision(ttg):
    # option validation happens before any device work
    import numpy as np
    t = [np.ones((1, 2, 1))]
    for opts in (ttg.RoundOptions(schedule=7), ttg.RoundOptions(precision=5),
                 ttg.RoundOptions(eps=-1.0)):
        with pytest.raises(ttg.TTGError) as e:
            ttg.round(t, opts)
        assert e.value.status == 1  # TTG_ERR_ARG


def test_no_silent_cpu_fallback(ttg):
    """Without a usable device every compute entry point fails with
    TTG_ERR_CUDA instead of computing on the host."""
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    import numpy as np
    with pytest.raises(ttg.TTGError) as e:
        ttg.round([np.ones((1, 2, 2)), np.ones((2, 2, 1))], ttg.RoundOptions(eps=1e-8))
    assert e.value.status == 9


def test_frob_norm_apply_argument_checks(ttg):
    # check_matvec_compatible / check_matmat_compatible run before any
    # device work; d = 0 is ||A x|| = 0 (tt_matrix_frob_norm_apply.hpp:38-41)
    import numpy as np
    A = [np.ones((1, 2, 3, 1))]
    with pytest.raises(ttg.TTGError) as e:
        ttg.frob_norm_apply(A, [np.ones((1, 2, 1))])      # mode mismatch (3 vs 2)
    assert e.value.status == 2
    with pytest.raises(ttg.TTGError) as e:
        ttg.frob_norm_apply([np.ones((1, 3, 1))], [np.ones((1, 3, 1))])   # A not a TT-matrix
    assert e.value.status == 1
    with pytest.raises(ttg.TTGError) as e:
        ttg.frob_norm_apply(A + A, [np.ones((1, 3, 1))])  # d mismatch
    assert e.value.status == 2
    assert ttg.frob_norm_apply([], []) == 0.0


def test_no_silent_cpu_fallback_new_entries(ttg):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    import numpy as np
    t = [np.ones((1, 2, 2)), np.ones((2, 2, 1))]
    for call in (lambda: ttg.soft_threshold(t, 0.5), lambda: ttg.left_orthogonalize(t),
                 lambda: ttg.frob_norm_apply([np.ones((1, 2, 2, 1))], [np.ones((1, 2, 1))])):
        with pytest.raises(ttg.TTGError) as e:
            call()
        assert e.value.status == 9


def test_shape_errors_before_device_work(ttg):
    # types/tt.hpp:35-70 (r_0 = r_d = 1, matching bonds) and
    # detail/shape_check.hpp: an invalid TT is refused whether or not a
    # device is present
    import numpy as np
    bad_bond = [np.ones((1, 2, 3)), np.ones((2, 2, 1))]     # 3 vs 2 at bond 1
    bad_r0 = [np.ones((2, 2, 1))]
    bad_rd = [np.ones((1, 2, 2))]
    for t in (bad_bond, bad_r0, bad_rd):
        for call in (lambda: ttg.round(t, ttg.RoundOptions(eps=1e-8)),
                     lambda: ttg.round_batch([t], ttg.RoundOptions(eps=1e-8)),
                     lambda: ttg.right_orthogonalize(t),
                     lambda: ttg.left_orthogonalize(t),
                     lambda: ttg.soft_threshold(t, 0.5),
                     lambda: ttg.inner(t, t)):
            with pytest.raises(ttg.TTGError) as e:
                call()
            assert e.value.status == 2, e.value
