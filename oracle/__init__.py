"""CPU oracle (test infrastructure): restatement of the reference's implicit
Beam_1 path in C, plus the recipe that builds the reference's own sources for
pinning.  Loaded only by tests/, the smoke check and bench.py's CPU legs."""
