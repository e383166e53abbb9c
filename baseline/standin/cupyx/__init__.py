"""Stand-in for cupyx (maps to SciPy); golden-vector generation only."""
