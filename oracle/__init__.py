"""CPU oracle for the Livre hot path (test infrastructure only; see oracle.h)."""
