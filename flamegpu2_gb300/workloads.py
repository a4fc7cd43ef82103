"""Benchmark workloads other than the default Boids line (see bench.py)."""


def run(name, args, world, rank, local):
    raise SystemExit(f"workload {name} is not available yet")
