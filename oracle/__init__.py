"""CPU oracle of the AxiSEM time loop -- test infrastructure only (see axisem_oracle.c)."""
