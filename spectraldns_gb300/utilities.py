"""Timer, memory and profile helpers with the interface of spectralDNS/utilities
(Timer __init__.py:18-68, MemoryUsage memoryprofiler.py:18-41,
create_profile create_profile.py:10-74) for a single process."""
import os
import time
from time import perf_counter


class Timer:
    """Fastest and slowest time step (spectralDNS/utilities/__init__.py:18-68)."""

    def __init__(self):
        self.fastest_timestep = 1e8
        self.slowest_timestep = 0
        self.t0 = perf_counter()
        self.tic = self.t0

    def __call__(self):
        t = perf_counter()
        dt = t - self.t0
        self.fastest_timestep = min(dt, self.fastest_timestep)
        self.slowest_timestep = max(dt, self.slowest_timestep)
        self.t0 = t

    def final(self, verbose=True):
        toc = perf_counter() - self.tic
        if verbose:
            print("Time = {}".format(toc))
            print("Fastest = {}".format(self.fastest_timestep))
            print("Slowest = {}".format(self.slowest_timestep))
        return toc


class MemoryUsage:
    """Resident set size of the process, printed with a label."""

    def __init__(self, s=""):
        self.memory = self._rss()
        self.first = self.memory
        if s:
            print(s, self.memory, "MB")

    @staticmethod
    def _rss():
        try:
            with open("/proc/self/statm") as f:
                return int(f.read().split()[1]) * os.sysconf("SC_PAGE_SIZE") / 1024 ** 2
        except Exception:
            return 0.0

    def __call__(self, s=""):
        self.prev = self.memory
        self.memory = self._rss()
        print("{0:26s}  {1:10.4f} MB {2:10.4f} MB".format(s, self.memory - self.prev, self.memory - self.first))


def reset_profile(prof):
    prof.code_map = {}
    prof.last_time = {}
    prof.enable_count = 0
    for func in getattr(prof, "functions", []):
        prof.add_function(func)


def create_profile(pr):
    """Digest of a cProfile.Profile for the solver's kernels (names as in the reference)."""
    import pstats
    import io
    s = io.StringIO()
    pstats.Stats(pr, stream=s).sort_stats("cumulative").print_stats(12)
    return {"report": s.getvalue()}
