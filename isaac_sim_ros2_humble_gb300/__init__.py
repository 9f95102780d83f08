"""GB300-native motion-planning hot path: FK, sphere collision, edge validation and
parallel RRT-Connect kernels behind a C-ABI (libgbmp)."""
