"""The engine's autotuner: picks the cell reach and the neighbour-list skin of
a handle, then the launch shape of the force pass (lanes per particle and
128-row blocks per CTA), then the lanes per particle of the density pass over
the kept lists, by timing each choice on the handle's current state, and
caches the choice per GPU model and workload signature in a JSON file.

No choice changes the pair sets (they are exact), and the fixed-point sums
make the reach and the launch shape irrelevant to the results; a skin changes
them only by the FP32 rounding of cell-local coordinates. So tuning is safe
to run on the production state itself: the steps it times are ordinary steps.
"""
import json
import math
import os

# (reach, skin); liquids, which diffuse fast, do best near skin 0.35 (fewer
# rebuilds for longer kept lists), membranes near 0.15 - 0.2
DEFAULT_CHOICES = ((1, 0.0), (2, 0.0), (1, 0.1), (1, 0.15), (1, 0.2), (1, 0.25), (1, 0.3),
                   (1, 0.35), (2, 0.15), (2, 0.2), (2, 0.3))
# (lanes per particle, row blocks per CTA) of the force pass; the first is the default
SHAPES = ((16, 1), (8, 1), (32, 1), (8, 2), (16, 2), (4, 1), (4, 2))
# lanes per particle of the density pass over kept lists; the first is the default
DENS_LANES = (32, 16, 8, 4)


def default_cache_path():
    """IDPD_TUNING_CACHE, else ~/.cache/implicit_dpd_gb300/tuning.json."""
    env = os.environ.get("IDPD_TUNING_CACHE")
    if env:
        return env
    return os.path.join(os.path.expanduser("~"), ".cache", "implicit_dpd_gb300", "tuning.json")


def signature(gpu, n_particles, volume, form, n_replicas=1):
    """Cache key: GPU model, pair-force form, replica count, particle count
    and number density rounded to a quarter octave (systems that close tune
    alike)."""
    q = lambda x: round(4.0 * math.log2(max(x, 1e-12))) / 4.0
    return f"{gpu}|form{form}|rep{n_replicas}|n2^{q(n_particles):g}|rho2^{q(n_particles / volume):g}"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, table):
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tune(engine, choices=DEFAULT_CHOICES, steps=40, key=None, cache_path=None, refresh=False,
         shapes=SHAPES, dens_lanes=DENS_LANES, rounds=2):
    """Applies the fastest (reach, skin), then the fastest force-pass shape
    (lanes, blocks) at that (reach, skin), then the fastest density-pass lanes
    (with kept lists), to `engine` and returns (choice, times): choice =
    {"reach", "skin", "lanes", "blocks", "dens_lanes"}, times maps
    "reach{r}_skin{s}", "lanes{l}_blocks{b}" and "dens_lanes{l}" to ms per
    step (empty when the choice came from the cache). With a key and a cache
    path, a cached choice is applied without timing unless refresh is set,
    and a new choice is written back. Choices whose skin the box does not
    allow are skipped; the launch shapes and the density lanes are timed
    `rounds` times each, in rounds over the candidates, keeping the fastest."""
    table = _load(cache_path) if (cache_path and key) else {}
    if key and not refresh and key in table:
        c = table[key]
        choice = {"reach": c["reach"], "skin": c["skin"], "lanes": c.get("lanes", shapes[0][0]),
                  "blocks": c.get("blocks", shapes[0][1]),
                  "dens_lanes": c.get("dens_lanes", dens_lanes[0])}
        engine.set_tuning(choice["reach"], choice["skin"], lanes=choice["lanes"],
                          blocks=choice["blocks"], dens_lanes=choice["dens_lanes"])
        return choice, {}

    def timed():
        engine.step(2)
        engine.step(steps)
        return engine.last_step_ms() / steps

    lanes0, blocks0 = shapes[0]
    dl0 = dens_lanes[0]
    times = {}
    for reach, skin in choices:
        try:
            engine.set_tuning(reach, skin, lanes=lanes0, blocks=blocks0, dens_lanes=dl0)
        except Exception:  # the box is too small for this skin
            continue
        times[(reach, skin)] = timed()
    if not times:
        raise ValueError("no tuning choice fits this system")
    reach, skin = min(times, key=times.get)
    # the launch shapes differ by a few per cent, about the spread of one
    # timing (the list rebuilds it catches): each is timed twice, in two
    # rounds over the candidates, and keeps its faster time
    shape_times = {}
    for _ in range(rounds):
        for lanes, blocks in shapes:
            engine.set_tuning(reach, skin, lanes=lanes, blocks=blocks, dens_lanes=dl0)
            t = timed()
            shape_times[(lanes, blocks)] = min(t, shape_times.get((lanes, blocks), t))
    lanes, blocks = min(shape_times, key=shape_times.get)
    dens_times = {dl0: shape_times[(lanes, blocks)]}
    if skin > 0:  # the density pass's lanes act on the kept lists only
        for _ in range(rounds):
            for dl in dens_lanes:
                engine.set_tuning(reach, skin, lanes=lanes, blocks=blocks, dens_lanes=dl)
                t = timed()
                dens_times[dl] = min(t, dens_times.get(dl, t))
    dl = min(dens_times, key=dens_times.get)
    engine.set_tuning(reach, skin, lanes=lanes, blocks=blocks, dens_lanes=dl)
    choice = {"reach": reach, "skin": skin, "lanes": lanes, "blocks": blocks, "dens_lanes": dl}
    if cache_path and key:
        table[key] = dict(choice, ms_per_step=dens_times[dl])
        _store(cache_path, table)
    out = {f"reach{r}_skin{s:g}": t for (r, s), t in times.items()}
    out.update({f"lanes{l}_blocks{b}": t for (l, b), t in shape_times.items()})
    out.update({f"dens_lanes{l}": t for l, t in dens_times.items()})
    return choice, out
