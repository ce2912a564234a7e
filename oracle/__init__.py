"""CPU parity checkers for the Analytic Marching engine -- test infrastructure
only (see am_oracle.h)."""
