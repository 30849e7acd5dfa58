"""Programs and loaders built from the reference's own sources (test
infrastructure only): fixture generators (ref_fixtures.cu, ref_partition.cu)
and the reference's SpMV kernels as a cubin (ref_kernels.cu, ref_gpu.py)."""
import os

_REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def sources():
    """The reference's source tree: $LOOPS_REF if set, else a `reference`
    folder beside this repository's folder.  Present only where the
    fixtures and the reference cubin are built; nothing at run time on a GPU
    needs it."""
    return os.environ.get("LOOPS_REF") or os.path.normpath(
        os.path.join(_REPO, os.pardir, "reference"))


def have_sources():
    return os.path.isdir(os.path.join(sources(), "include", "loops"))
