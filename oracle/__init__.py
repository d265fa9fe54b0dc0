"""Oracle (test infrastructure): the reference build recipe and the C restatement."""
