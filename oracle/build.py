"""Build step for the oracle (test infrastructure only).

The oracle is a NumPy restatement of the reference (``turn_loop.py``) and
needs no compilation.  The reference itself is Python with one Cython
module; it is imported only in the container that holds its source tree,
to generate the golden fixtures (``tests/golden/make_golden.py`` builds it
in a scratch directory outside the repository).  It is not built into
``oracle/_ref``: a Python package cannot travel to the GPU host, so the
timed CPU baseline there is the NumPy port (``kind: port``).
"""


def build():
    """Nothing to compile; kept so that the build entry point states it."""
    return None
