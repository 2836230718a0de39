"""Python side of the GB300 sphere-DEM timestep: a ctypes binding of the C ABI
(``api``), its in-tree build (``build``) and seeded synthetic workloads
(``workloads``)."""
