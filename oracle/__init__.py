"""CPU oracle of LUE's flow-routing path.  Test infrastructure only; see lue_oracle.c."""
