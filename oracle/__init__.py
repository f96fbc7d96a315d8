"""Parity oracle package (test infrastructure only)."""
