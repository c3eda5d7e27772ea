"""CPU oracle for the nerf-tf2 render path. TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only as the checker. The product
path (the CUDA library and its Python mirror) never calls into it.

Parity unpinned: the reference is TensorFlow 2.6 Python code, TensorFlow is not
installed here and cannot be installed, and the reference ships no tests,
golden vectors or fixtures for this path. The oracle is a line-by-line
restatement of the reference's arithmetic, pinned only by closed-form
known-answer tests.
"""
from .nerf_oracle import *  # noqa: F401,F403
