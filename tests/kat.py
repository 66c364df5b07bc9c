"""The reference's known-answer tests, restated once for every method.

* acceleration_error: particular/src/gravity/newtonian/mod.rs:228-277
* circular_orbit:     particular/src/gravity/newtonian/mod.rs:281-347

`compute(storage)` is any compute method's entry: it receives a storage (a
Reordered, or a packed (n, 4) float32 array for the orbit) and returns the
(n, 3) accelerations of the affected bodies.
"""
import numpy as np

from particular_gb300 import Reordered


def acceleration_error(compute, epsilon):
    s = np.float32
    massive = [((0.0,) * 3, 20.0), ((1.0,) * 3, 30.0), ((-3.0,) * 3, 40.0)]
    particles = [((10.0,) * 3, 0.0), massive[0], massive[1], massive[2], ((30.0,) * 3, 0.0),
                 ((-45.0,) * 3, 0.0)]
    reordered = Reordered(particles)  # is_affecting: m != 0
    computed = np.asarray(compute(reordered), np.float32)
    assert computed.shape == (6, 3)
    errors = []
    for k, (pos1, _m1) in enumerate(particles):
        acc = np.zeros(3, np.float32)
        for pos2, m2 in massive:
            d = np.asarray(pos2, s) - np.asarray(pos1, s)
            mag2 = s(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
            if mag2 != 0:
                acc = acc + d * s(m2) * np.sqrt(s(1.0) / mag2) / mag2
        err = float(np.sqrt(((s(1.0) - computed[k] / acc) ** 2).sum()))
        errors.append(err)
        assert err <= epsilon, (k, computed[k], acc, err)
    return errors


def circular_orbit(compute, orbit_count, epsilon):
    s = np.float32
    DT = s(1.0 / 60.0)
    parts = np.zeros((2, 4), s)
    parts[0, 3] = 1e6
    parts[1, 0] = 100.0
    vel = np.zeros((2, 3), s)
    vel[1, 1] = 100.0

    def dist():
        d = parts[0, :3] - parts[1, :3]
        return s(np.sqrt(s(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])))

    def energy(r):
        return -(parts[0, 3] + parts[1, 3]) / (r + r)

    d0 = dist()
    e0 = energy(d0)
    period = s(2.0 * np.pi) * np.sqrt((d0 * d0 * d0) / parts[0, 3])
    steps = int(round(float(period / DT)))
    for _ in range(steps * orbit_count):
        a = np.asarray(compute(parts), s)
        vel += a * DT
        parts[:, :3] += vel * DT
    d1 = dist()
    e1 = energy(d1)
    err_d = abs(1.0 - float(d0 / d1))
    err_e = abs(1.0 - float(e0 / e1))
    assert err_d < epsilon, err_d
    assert err_e < epsilon, err_e
    return err_d, err_e
