"""Loader of the optional libtorch binding (torch_ext/pp_cumsum.cpp): a
differentiable float32 cumsum along the last dimension whose forward and
backward run the library's row-scan kernels through the C ABI.

    import ppcumsum
    ext = ppcumsum.load()
    y = ext.cumsum(x)            # x: float32 CUDA tensor, requires_grad ok
    y.backward(g)                # x.grad = suffix sums of g along the last dim
"""

from __future__ import annotations

from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent

_ext = None


def load(verbose: bool = False):
    """Build (once, into _build/torch_ext) and import the extension."""
    global _ext
    if _ext is not None:
        return _ext
    from torch.utils.cpp_extension import CUDA_HOME
    from torch.utils.cpp_extension import load as _load

    import ppbuild

    lib = ppbuild.build()
    build_dir = PKG / "_build" / "torch_ext"
    build_dir.mkdir(parents=True, exist_ok=True)
    _ext = _load(
        name="pp_cumsum_ext",
        sources=[str(PKG / "torch_ext" / "pp_cumsum.cpp")],
        extra_include_paths=[str(ROOT / "include"), str(Path(CUDA_HOME or "/usr/local/cuda") / "include")],
        extra_ldflags=[str(lib), f"-Wl,-rpath,{lib.parent}"],
        extra_cflags=["-O2"],
        build_directory=str(build_dir),
        verbose=verbose,
    )
    return _ext
