"""Oracle for libbhgpu's parity tests (test infrastructure only; see oracle.py)."""
