"""CPU oracle (test infrastructure): a numpy restatement of the reference's algorithm."""
