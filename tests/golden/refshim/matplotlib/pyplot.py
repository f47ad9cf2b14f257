"""Empty stand-in so PETITE's plot-only import succeeds (see README.txt)."""
