"""Test infrastructure: CPU oracle for the BC7 encoder (never product code)."""
