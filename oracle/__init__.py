"""CPU oracle package (test infrastructure; see oracle.py)."""
