"""CPU oracle for the D3Q19 hot path (test infrastructure only; see oracle.py)."""
