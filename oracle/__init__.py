"""CPU oracle for the soil/snow column solve — test infrastructure only (see clm_oracle.c)."""
