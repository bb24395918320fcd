"""GB300 hair-physics step: host-side mirror of the C ABI in include/rvh.h."""
