"""Measurement probes of bench.py and the tests (libctraj_probes.so); not part of the engine."""
