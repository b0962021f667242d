"""CPU oracle of the LightFEM solve path: test infrastructure only (see lf_oracle.cpp)."""
