"""Import the real reference package (qaravan) where its source tree is present.

TEST INFRASTRUCTURE ONLY. Used by ``tests/golden/make_golden.py`` and by the
CPU cross-checks in ``tests/`` that are skipped when the reference is absent.

The reference imports three packages that are not installed here:
``ncon_torch`` (all contraction arithmetic; served by ``oracle.ncon``),
``matplotlib`` (imported only by ``core/lattices.py:2``) and ``stim``
(imported only by ``algebraQ/clifford_sim.py:3``). Empty stand-ins for the
last two and a forwarding ``ncon_torch`` module are written to a temporary
directory placed on ``sys.path``; nothing is written into the reference tree
(``sys.dont_write_bytecode`` is set while importing).
"""
from __future__ import annotations

import os
import sys
import tempfile

REF_SRC = os.environ.get("QGB_REFERENCE_SRC", "/root/reference/src")

_STUBS = {
    "ncon_torch/__init__.py": "from oracle.ncon import ncon, permute\n",
    "matplotlib/__init__.py": "",
    "matplotlib/pyplot.py": "def __getattr__(name):\n    raise AttributeError(name)\n",
    "stim/__init__.py": "",
}

_cached = None


def available() -> bool:
    return os.path.isdir(os.path.join(REF_SRC, "qaravan"))


def load():
    """Return the imported ``qaravan`` module (tensorQ and core star-imported)."""
    global _cached
    if _cached is not None:
        return _cached
    if not available():
        raise RuntimeError(f"reference source tree not found at {REF_SRC}")
    stub_dir = tempfile.mkdtemp(prefix="qgb_refstubs_")
    for rel, text in _STUBS.items():
        path = os.path.join(stub_dir, rel)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            f.write(text)
    repo_root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (repo_root, stub_dir, REF_SRC):
        if p not in sys.path:
            sys.path.insert(0, p)
    old = sys.dont_write_bytecode
    sys.dont_write_bytecode = True
    try:
        import qaravan  # noqa: F401
        import qaravan.core as core
        import qaravan.tensorQ as tq
    finally:
        sys.dont_write_bytecode = old

    class _Ref:
        pass

    ref = _Ref()
    ref.core = core
    ref.tensorQ = tq
    _cached = ref
    return ref
