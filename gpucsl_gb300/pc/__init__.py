"""Public API of the skeleton-discovery path, laid out like the reference's gpucsl.pc."""
