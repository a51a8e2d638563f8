"""fdtomoc_gb300 — GB300-native spherical finite-difference travel-time solver (FDtomoC sphfd)."""
