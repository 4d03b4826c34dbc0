"""CPU oracle for the RT solve -- test infrastructure only (see rt_oracle.py)."""
