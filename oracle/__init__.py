"""CPU oracle package (test infrastructure only; see cs_oracle.h)."""
