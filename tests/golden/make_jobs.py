"""Generate the batched-jobs fixture (64 jobs, seed 1) and the serving stream (seed 2).

    python tests/golden/make_jobs.py

jobs_config4.json: for each of 64 jobs, drawn in order from
numpy.random.default_rng(1): n_start ~ U[1e3, 1e6], n_width ~ logU[1e3, 1e5],
p_start ~ logU[max(n_end, 1e9), 2^62], p_width ~ logU[1e7, 1e9]
(the four draws of a job are consecutive; integer parts are kept).

stream_config5.json: Poisson arrivals, mean 20/s for 120 s, from
numpy.random.default_rng(2): exponential inter-arrival gaps, and for each
arrival a job drawn from the same distribution as jobs_config4.json with the
same generator (so the stream is reproducible from the seed alone).
"""
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def draw_job(rng):
    n_start = int(rng.uniform(1e3, 1e6))
    n_width = int(math.exp(rng.uniform(math.log(1e3), math.log(1e5))))
    n_end = n_start + n_width
    lo = max(n_end, 1e9)
    p_start = int(math.exp(rng.uniform(math.log(lo), math.log(2.0**62))))
    p_width = int(math.exp(rng.uniform(math.log(1e7), math.log(1e9))))
    return [p_start, p_start + p_width, n_start, n_end]


def jobs_config4():
    rng = np.random.default_rng(1)
    return [draw_job(rng) for _ in range(64)]


def stream_config5(rate=20.0, duration=120.0):
    rng = np.random.default_rng(2)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        out.append([round(t, 6)] + draw_job(rng))
    return out


if __name__ == "__main__":
    with open(os.path.join(HERE, "jobs_config4.json"), "w") as fh:
        json.dump({"seed": 1, "columns": ["pmin", "pmax", "nmin", "nmax"], "jobs": jobs_config4()}, fh)
    s = stream_config5()
    with open(os.path.join(HERE, "stream_config5.json"), "w") as fh:
        json.dump({"seed": 2, "rate_per_s": 20.0, "duration_s": 120.0,
                   "columns": ["arrival_s", "pmin", "pmax", "nmin", "nmax"], "requests": s}, fh)
    print(len(jobs_config4()), "jobs;", len(s), "requests")
