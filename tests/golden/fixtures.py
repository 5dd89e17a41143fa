"""Small seeded parity fixtures (oracle outputs) for the GPU tests."""


def write_all(out_dir):
    """Fixtures are added next to the CUDA paths they check."""
    return out_dir
