"""CPU oracle for the GPUGraphs.jl semiring kernels and graph algorithms.

Test infrastructure only: tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg use it as the checker; the product never imports it."""
