"""CPU oracle of the BEHF time stepper -- test infrastructure (the checker), never the product path."""
