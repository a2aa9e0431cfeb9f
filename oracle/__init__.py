"""CPU oracle for the fluid step (test infrastructure only; see fs_oracle.h)."""
