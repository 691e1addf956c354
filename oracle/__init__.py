"""CPU restatement of the reference path (test infrastructure only; see vt_oracle.h)."""
