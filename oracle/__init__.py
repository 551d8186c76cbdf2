"""Test infrastructure: the CPU oracle of the ray-query engine (see oracle.h)."""
