"""CPU FP64 oracle (test infrastructure only; see crtm_oracle.h)."""
