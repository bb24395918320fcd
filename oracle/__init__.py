"""CPU oracle of the hair step: TEST INFRASTRUCTURE ONLY (tests/, smoke(), bench.py CPU legs)."""
