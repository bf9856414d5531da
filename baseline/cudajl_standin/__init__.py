"""Comparator arm only: an unfused FP64 restatement of FourierFlows.jl's GPU path (CUDA.jl
broadcasts + CUFFT), timed beside the library's fused step by bench.py and checked
against the oracle by the tests.  Not part of the library."""
