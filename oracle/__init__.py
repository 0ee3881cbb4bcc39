"""Checkers for the FDTD product (TEST INFRASTRUCTURE ONLY): the CPU oracle restating the
reference scheme, its build recipe, and the launcher for the reference's own kernels."""
