"""The C++ mirror of the reference API (include/nscale_gpu.hpp) compiles and links against the
library with the reference's call-site forms (no GPU needed to build)."""
import os

import pytest

from cpp_api import build, LIBDIR


def test_cpp_api_builds(tmp_path):
    if not os.path.exists(os.path.join(LIBDIR, "libnsgb.so")):
        pytest.skip("library not built")
    exe = tmp_path / "nscale_api_test"
    build(str(exe))
    assert exe.exists()
