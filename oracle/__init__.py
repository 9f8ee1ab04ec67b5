"""CPU restatement of illume's path tracer (test infrastructure only; see oracle.h)."""
