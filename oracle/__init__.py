"""Oracle package: CPU restatement of the reference's hot path and access to the
reference's own code.  TEST INFRASTRUCTURE ONLY -- imported by tests/, the smoke
check and bench.py's CPU-baseline / reference legs, never by the product."""
