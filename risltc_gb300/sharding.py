"""Pixel partitioning across ranks.

Every pixel of the shading pass is independent (shading_pass.frag.glsl:674-770
reads only per-pixel inputs and read-only scene data), so a frame splits into
contiguous row bands with no exchange during shading; only the finished bands
are gathered.
"""


def row_band(rank, world, height):
    """Rows [begin, end) of the frame shaded by `rank` of `world`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside world of %d" % (rank, world))
    base, extra = divmod(height, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)
