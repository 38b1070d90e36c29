"""Mirror of the reference's ``fast_em`` package (fast_em/laml.py,
fast_em/calculations.py, fast_em/phylogeny.py) running on the GB300 engine."""
