"""CPU oracle of the transport (test infrastructure; see mc_oracle.cpp)."""
