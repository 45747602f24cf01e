"""CPU oracle for parity tests -- TEST INFRASTRUCTURE ONLY (see oracle/oracle.py)."""
