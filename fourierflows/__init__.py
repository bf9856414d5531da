"""Namespace of the FourierFlows ports; the GB300 build is ``fourierflows.jl_gb300``."""
