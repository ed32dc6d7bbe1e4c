"""CPU oracle of the coupled step (test infrastructure; see pf_oracle.c)."""
