"""Programs and loaders built from the reference's own sources (test
infrastructure only): fixture generators (ref_fixtures.cu, ref_partition.cu)
and the reference's SpMV kernels as a cubin (ref_kernels.cu, ref_gpu.py)."""
