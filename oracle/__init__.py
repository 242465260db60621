"""Test infrastructure: the CPU oracle of the wavetorch time-stepping path."""
