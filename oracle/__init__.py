"""CPU oracle of the HORAYZON horizon / sky-view-factor path.

TEST INFRASTRUCTURE. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` import this package, as the checker of the
CUDA path. The product package ``horayzon_extpar_gb300`` never imports it.

* ``hz_oracle.c`` restates mo_lradtopo_horayzon.cpp in C (FP32 reference
  semantics and an FP64 variant), built into ``oracle/_build/``.
* ``shim/`` + ``ref_entry.cpp`` compile the unmodified reference source
  against project-written Embree/TBB stand-ins into ``oracle/_ref/`` when the
  reference tree is available.
"""
