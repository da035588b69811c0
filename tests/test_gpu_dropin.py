"""The module swap of the drop-in, replayed on the GPU.

tests/golden/seam_calls.json holds every call that the reference's own
perm.matrix_permanent, perm.permanent and perm_binary.binary_permanent made
through their native seams (perm.py:917-923, 752-753; perm_binary.py:822-824)
while computing the recorded results, with the compiled extensions' return
values (tests/golden/make_seam_calls.py).  Installing permgpu.GpuExt as
perm.perm_c_ext (and BinaryGpuExt as perm_binary._binary_ext) is transparent
exactly when the GPU objects return the recorded value for every recorded
call: the reference's Python code then takes the same path and reaches the
same result.  The results themselves are checked against the whole-call
GPU API too.
"""

import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def test_recorded_seam_calls_replay_on_the_gpu_objects(lib):
    import permgpu
    from permgpu.ext import BinaryGpuExt, GpuExt
    ext, bext = GpuExt(), BinaryGpuExt()
    data = golden("seam_calls.json")
    replayed = 0
    for case in data["cases"]:
        for call in case["calls"]:
            target = bext if call["fn"] == "binary_permanent_mod_p" else ext
            assert getattr(target, call["fn"])(*call["args"]) == call["result"], \
                (case["api"], call["fn"])
            replayed += 1
        want = int(case["result"])
        if case["api"] == "perm.matrix_permanent":
            assert permgpu.matrix_permanent(case["matrix"], method="generic") == want
        elif case["api"] == "perm.permanent":
            assert permgpu.permanent(case["n"]) == want
        else:
            assert permgpu.binary_permanent(case["matrix"]) == want
    assert replayed >= 20
