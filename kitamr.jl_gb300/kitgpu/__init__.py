"""Host side of the GB300 implementation of KitAMR.jl's per-step phase-space hot path."""
