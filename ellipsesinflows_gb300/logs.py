"""The reference's log files (src/logging.c:197-208) from the device reductions.

``LogWriter(sim, rate).write()`` appends one line per file at the solver's current
step and time, in the reference's formats and file names under ``dirname``
(default ``output/log``, FILEIO_LOG of include/fileio.h):

    progress.dat        step, time, dt               (show_progress, :21-38)
    divergence.dat      time, max |div u|, sum div u (check_divergence, :40-85)
    momentum.dat        time, x and y momentum       (check_momentum, :87-128)
    energy.dat          time, x and y kinetic energy (check_energy, :130-172)
    particle%010d.dat   time, x, y, az, ux, uy, vz   (check_particle, :174-195)

The field sums come from one device pass (eif_log_quantities); only the particle
records are copied to the host. Files are created at step 0 and appended to
afterwards, as in the reference. The progress line is also printed.
"""
import os


def ndigits(rate):
    """get_ngidits (src/logging.c:12-19): digits after the point of the time column"""
    n = 1
    inv = int(1.0 / rate)
    while True:
        inv = int(inv / 10)
        if inv == 0:
            return n
        n += 1


class LogWriter:
    def __init__(self, sim, rate, dirname=os.path.join("output", "log"), echo=True):
        self.sim, self.rate, self.dirname, self.echo = sim, float(rate), dirname, echo

    def _open(self, name, step):
        os.makedirs(self.dirname, exist_ok=True)
        return open(os.path.join(self.dirname, name), "w" if step == 0 else "a")

    def write(self):
        sim = self.sim
        step, time = sim.time_state()
        dt = sim.dt
        q = sim.log_quantities()
        rec = sim.pull_particles()
        nd = ndigits(self.rate)
        line = "step %8d, time %*.*f, dt %.2e\n" % (step, nd + 3, nd, time, dt)
        with self._open("progress.dat", step) as f:
            f.write(line)
        if self.echo:
            print(line, end="")
        with self._open("divergence.dat", step) as f:
            f.write("%*.*f % .1e % .1e\n" % (nd + 3, nd, time, q["divmax"], q["divsum"]))
        with self._open("momentum.dat", step) as f:
            f.write("%*.*f % 18.15e % 18.15e\n" % (nd + 3, nd, time, q["momentum"][0], q["momentum"][1]))
        with self._open("energy.dat", step) as f:
            f.write("%*.*f % 18.15e % 18.15e\n" % (nd + 3, nd, time, q["energy"][0], q["energy"][1]))
        from .capi import F
        for n in range(rec.shape[0]):
            r = rec[n]
            with self._open("particle%010d.dat" % n, step) as f:
                f.write("%*.*f % .7e % .7e % .7e % .7e % .7e % .7e\n" % (
                    nd + 3, nd, time, r[F["x"]], r[F["y"]], r[F["az"]], r[F["ux"]], r[F["uy"]], r[F["vz"]]))
