"""bench.py's host-side helpers on the CPU: the central-difference check's skip and
Richardson logic on functions with known derivatives, and JSON output of numpy values."""
import json

import numpy as np

import bench


def test_fd_check_accepts_smooth_and_skips_kinks():
    rng = np.random.default_rng(0)
    xs = np.linspace(1.0, 2.0, 50)

    def draw():
        c = int(rng.integers(0, 50))
        return "s", 0, (c, 0, 0), float(xs[c])

    # J(x) = x^3 summed per entry: dJ/dx = 3 x^2
    smooth = bench.fd_check(lambda f, c, cell: np.float64(3 * xs[cell[0]] ** 2),
                            lambda f, c, cell, h: (xs[cell[0]] + h) ** 3 - (xs[cell[0]] - h) ** 3,
                            draw, 20, 40)
    assert smooth["entries"] == 20 and smooth["skipped_limiter_switch"] == 0
    assert smooth["worst_rel_err"] < 1e-9 and smooth["passed"] is True
    # J = |x - x_k| with the kink x_k = x (1 + 3e-7) inside [x - h/2, x + h/2]: the two
    # quotients disagree, and every entry is skipped

    def jdiff_kink(f, c, cell, h):
        x = xs[cell[0]]
        xk = x * (1 + 3e-7)
        return abs(x + h - xk) - abs(x - h - xk)

    kink = bench.fd_check(lambda f, c, cell: np.float64(1.0), jdiff_kink, draw, 5, 10)
    assert kink["entries"] == 0 and kink["skipped_limiter_switch"] == 10 and kink["passed"] is False
    json.dumps(smooth, default=bench.jsonable)
    json.dumps(kink, default=bench.jsonable)


def test_jsonable_numpy_values():
    line = {"a": np.float64(1.5), "b": np.bool_(True), "c": np.arange(3), "d": np.int32(4)}
    assert json.loads(json.dumps(line, default=bench.jsonable)) == {"a": 1.5, "b": True, "c": [0, 1, 2], "d": 4}
