"""Autotuner for the batched form: particles per CTA, shared tile capacity and P2G flush strategy.

Every setting produces the same bits (the grid sums are integers and each particle's update is
independent), so the tuner times real substeps of the world's own scenes: the substeps it runs
are part of the simulation, not a separate benchmark. For each candidate it runs `substeps`
substeps `repeats` times between timing marks on the world's stream and keeps the fastest median.

Candidates (the reference has no such knobs; its tile capacity follows the device limit,
src/physics/mpm.js:298-302):
  particles per CTA  256, 512, 1024       (one, two or four particles per thread)
  tile capacity      343 (7^3: the stencil box of one 4^3 sort block), 1331 (11^3: of an 8^3 box),
                     2048 (the largest the shared tile holds)
  flush              0 = shared tile, non-zero nodes flushed with global i32 atomics
                     1 = global i32 atomics per particle and node
"""
import itertools
import statistics

PARTICLES_PER_CTA = (256, 512, 1024)
TILE_NODES = (343, 1331, 2048)
FLUSH = (0, 1)


def candidates():
    return list(itertools.product(PARTICLES_PER_CTA, TILE_NODES, FLUSH))


def time_substeps(world, substeps, repeats):
    """Median GPU ms of world.step(substeps) over `repeats` runs (after one untimed run)."""
    world.step(substeps)
    out = []
    for _ in range(repeats):
        world.mark(6)
        world.step(substeps)
        world.mark(7)
        out.append(world.elapsed(6, 7))
    return statistics.median(out)


def autotune(world, substeps=4, repeats=3, cands=None, log=None):
    """Tries each (particles_per_cta, tile_nodes, flush) on `world`, applies and returns the fastest
    as a dict with the per-candidate timings (ms per substep)."""
    results = {}
    for ppc, tile, flush in (cands or candidates()):
        world.set_tuning(ppc, tile, flush)
        ms = time_substeps(world, substeps, repeats) / substeps
        results[(ppc, tile, flush)] = ms
        if log:
            log(f"autotune ppc={ppc} tile={tile} flush={flush}: {ms * 1e3:.1f} us/substep")
    best = min(results, key=results.get)
    world.set_tuning(*best)
    return {"particles_per_cta": best[0], "tile_nodes": best[1], "flush": best[2],
            "ms_per_substep": results[best],
            "table": {f"{k[0]}/{k[1]}/{k[2]}": v for k, v in results.items()}}
