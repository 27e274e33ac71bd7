"""ORACLE — test infrastructure only.

Nothing in the product package (``matpl_gb300``) imports this package.  Only the tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use it, and only to check
results and as the CPU baseline, never as the thing measured on the GPU.

Contents
--------
``neighconst.c``   plain-C restatement of ``src/pre_data/gen_feature/NeighConst.f90:14-149``
``neigh.py``       ctypes loader + numpy glue reproducing ``dpuni_data_loader.find_neighbore``
``dp_oracle.py``   torch-FP64 restatement of ``src/model/dp_dp_script.py`` (DP se_e2_a E/F/V)
``build.py``       compiles ``neighconst.c`` (gcc, ``-ffp-contract=off``)
"""
