"""CPU oracle package: test infrastructure only (see ldm_oracle.py header)."""
