"""CPU oracle (test infrastructure only; see cr_oracle.h)."""
