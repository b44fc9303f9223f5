"""Reference-format output and checkpoint/resume.

State file: the text branch of PathIntegralMonteCarlo::saveState
(src/pimc.cpp:923-1000), read back as PathIntegralMonteCarlo::loadState does
(src/pimc.cpp:1108-1290):

    numWorldLines                              Path::getNumParticles (Ne)
    "%16d\\t%16d"  total accepted, attempted    first move's totals
    "%16d\\t%16d"  per move: accepted, attempted
    "%16d\\t%16d"  per estimator: totNumAccumulated, numSampled
    beads       DynamicArray<dVec,2> at precision 16
    nextLink    DynamicArray<beadLocator,2>
    prevLink
    worm.beads  DynamicArray<unsigned int,2>
    625 generator words, each followed by a space    MTRand::save

A 2-D array streams as "(0,R-1) x (0,C-1)\\n[ a b ... \\n  ... ]\\n" with a
std::array as "(x,y,z)" (include/common.h:245-274); the saver adds one more
newline after each array.  Doubles print as iostream's default float format
at precision 16, which is C's "%.16g".

Estimator files (src/estimator.cpp:260-410, src/communicator.cpp:39-46,
158-170): OUTPUT/<ensemble>-<label>-<dataName>.dat, a header line written
only when the run is not a restart or the file is new, then one row of
"%16.8E" columns per bin, each the bin sum times its norm over the number of
accumulated samples.
"""
import io
import json
import os
import re

import numpy as np

MT_SAVE_WORDS = 625                  # MTRand::SAVE = N + 1 (MersenneTwister.h)
NO_BEAD = -1                         # XXX, include/common.h:93


# --------------------------------------------------------------------------
# state file
# --------------------------------------------------------------------------
def _g16(x):
    return "%.16g" % x


def _array2(rows, cols, cell):
    """One 2-D DynamicArray in the stream format of include/common.h:258-274."""
    out = io.StringIO()
    out.write("(0,%d) x (0,%d)\n[ " % (rows - 1, cols - 1))
    for i in range(rows):
        for j in range(cols):
            out.write(cell(i, j))
            out.write(" ")
        if i < rows - 1:
            out.write("\n  ")
    out.write("]\n")
    return out.getvalue()


def left_pack(cfg):
    """Path::leftPack (src/path.cpp:145-189): move the active beads of every
    slice to the lowest particle indices, relinking their neighbours.
    Returns a new configuration dict; the input is not modified."""
    pos = np.array(cfg["pos"], dtype=np.float64, copy=True)
    nxt = np.array(cfg["next"], dtype=np.int32, copy=True)
    prv = np.array(cfg["prev"], dtype=np.int32, copy=True)
    on = np.array(cfg["on"], dtype=np.uint8, copy=True)
    m, ne = on.shape
    for t in range(m):
        for p in range(ne):
            if on[t, p]:
                continue
            q = next((k for k in range(p + 1, ne) if on[t, k]), None)
            if q is None:
                continue
            pos[t, p] = pos[t, q]
            on[t, p], on[t, q] = 1, 0
            nxt[t, p], prv[t, p] = nxt[t, q], prv[t, q]
            ps, pp = prv[t, q]
            ns, np_ = nxt[t, q]
            # next(prev(bead2)) = bead1; prev(next(bead2)) = bead1; a missing
            # neighbour (XXX) wraps to the last entry in the reference; here
            # an end of an open worldline simply has none
            if ps >= 0:
                nxt[ps, pp] = (t, p)
            if ns >= 0:
                prv[ns, np_] = (t, p)
            nxt[t, q] = NO_BEAD
            prv[t, q] = NO_BEAD
    out = dict(cfg)
    out.update(pos=pos, next=nxt, prev=prv, on=on)
    return out


def format_state(cfg, rng_words, move_counts=(), estimator_counts=(), total=None):
    """The state text of one path.

    cfg: pos [M][Ne][3], next/prev [M][Ne][2], on [M][Ne] (left-packed as
    saveState leaves them); rng_words: 625 MTRand::save words;
    move_counts: (accepted, attempted) per move, in the move list's order;
    estimator_counts: (totNumAccumulated, numSampled) per estimator; total:
    the first move's (totAccepted, totAttempted), by default the sums of
    move_counts."""
    pos = np.asarray(cfg["pos"], dtype=np.float64)
    nxt = np.asarray(cfg["next"], dtype=np.int64)
    prv = np.asarray(cfg["prev"], dtype=np.int64)
    on = np.asarray(cfg["on"]).astype(np.int64)
    m, ne = on.shape
    if pos.shape != (m, ne, 3) or nxt.shape != (m, ne, 2) or prv.shape != (m, ne, 2):
        raise ValueError("state: pos/next/prev must be [M][Ne][3|2] with on [M][Ne]")
    words = np.asarray(rng_words, dtype=np.uint64)
    if words.shape != (MT_SAVE_WORDS,):
        raise ValueError("state: the generator state has 625 words")
    if total is None:
        total = (sum(int(a) for a, _ in move_counts), sum(int(b) for _, b in move_counts))
    out = io.StringIO()
    out.write("%d\n" % ne)
    out.write("%16d\t%16d\n" % (int(total[0]), int(total[1])))
    for a, b in move_counts:
        out.write("%16d\t%16d\n" % (int(a), int(b)))
    for a, b in estimator_counts:
        out.write("%16d\t%16d\n" % (int(a), int(b)))
    out.write(_array2(m, ne, lambda i, j: "(%s,%s,%s)" % (_g16(pos[i, j, 0]), _g16(pos[i, j, 1]),
                                                           _g16(pos[i, j, 2]))))
    out.write("\n")
    out.write(_array2(m, ne, lambda i, j: "(%d,%d)" % (nxt[i, j, 0], nxt[i, j, 1])))
    out.write("\n")
    out.write(_array2(m, ne, lambda i, j: "(%d,%d)" % (prv[i, j, 0], prv[i, j, 1])))
    out.write("\n")
    out.write(_array2(m, ne, lambda i, j: "%d" % on[i, j]))
    out.write("\n")
    out.write("".join("%d " % int(w) for w in words))
    out.write("\n")
    return out.getvalue()


_HEADER = re.compile(r"\(\s*(-?\d+)\s*,\s*(-?\d+)\s*\)\s*x\s*\(\s*(-?\d+)\s*,\s*(-?\d+)\s*\)")


class _Reader:
    """Token reader with istream semantics: whitespace skipped, '(' ',' ')'
    read as single characters, numbers as the longest run of number chars."""

    def __init__(self, text):
        self.s, self.i = text, 0

    def ws(self):
        s, i = self.s, self.i
        while i < len(s) and s[i] in " \t\r\n":
            i += 1
        self.i = i

    def ch(self):
        self.ws()
        if self.i >= len(self.s):
            raise ValueError("state: unexpected end of file")
        c = self.s[self.i]
        self.i += 1
        return c

    def expect(self, c):
        got = self.ch()
        if got != c:
            raise ValueError("state: expected %r, found %r at offset %d" % (c, got, self.i - 1))

    _num = re.compile(r"[-+]?(?:\d+\.?\d*(?:[eE][-+]?\d+)?|\.\d+(?:[eE][-+]?\d+)?|inf|nan)",
                      re.IGNORECASE)

    def number(self):
        self.ws()
        mt = self._num.match(self.s, self.i)
        if not mt:
            raise ValueError("state: expected a number at offset %d" % self.i)
        self.i = mt.end()
        return mt.group(0)

    def line(self):
        j = self.s.find("\n", self.i)
        j = len(self.s) if j < 0 else j
        out = self.s[self.i:j]
        self.i = min(j + 1, len(self.s))
        return out

    def array2(self, cell):
        """operator>>(istream, DynamicArray<T,2>&), include/common.h:305-399."""
        self.ws()
        mt = _HEADER.match(self.s, self.i)
        if not mt:
            raise ValueError("state: expected an array header at offset %d" % self.i)
        r0, r1, c0, c1 = (int(g) for g in mt.groups())
        self.i = mt.end()
        while self.ch() != "[":
            pass
        rows, cols = r1 - r0 + 1, c1 - c0 + 1
        vals = [[cell(self) for _ in range(cols)] for _ in range(rows)]
        while self.ch() != "]":
            pass
        return vals


def _dvec(r):
    r.expect("(")
    x = float(r.number()); r.expect(",")
    y = float(r.number()); r.expect(",")
    z = float(r.number()); r.expect(")")
    return (x, y, z)


def _loc(r):
    r.expect("(")
    s = int(r.number()); r.expect(",")
    p = int(r.number()); r.expect(")")
    return (s, p)


def parse_state(text):
    """Every field of a state file: num_worldlines, the count lines
    (pairs of ints) before the beads, beads, next, prev, worm beads, rng."""
    r = _Reader(text)
    nwl = int(r.number())
    r.line()
    counts = []
    while True:                     # loadState skips to the first '(' line
        r.ws()
        if r.i >= len(r.s) or r.s[r.i] == "(":
            break
        ln = r.line().split()
        if ln:
            counts.append(tuple(int(v) for v in ln))
    beads = np.array(r.array2(_dvec), dtype=np.float64)
    nxt = np.array(r.array2(_loc), dtype=np.int32)
    prv = np.array(r.array2(_loc), dtype=np.int32)
    worm = np.array(r.array2(lambda rr: int(rr.number())), dtype=np.int64)
    words = []
    while len(words) < MT_SAVE_WORDS:
        r.ws()
        if r.i >= len(r.s):
            break
        words.append(int(r.number()))
    rng = np.array(words, dtype=np.uint32) if len(words) == MT_SAVE_WORDS else None
    return dict(num_worldlines=nwl, counts=counts, beads=beads, next=nxt, prev=prv,
                worm_beads=worm, rng=rng)


def _put_in_bc(r, side):
    side = np.asarray(side, dtype=np.float64)
    return r - side * np.floor(r * (1.0 / side) + 0.5)


def load_state(text, num_slices, side, restart=True):
    """The configuration a reference run starts from after loadState
    (src/pimc.cpp:1108-1290) for a fully periodic box.

    With the file's slice count equal to num_slices the arrays are taken as
    they are; otherwise every active slice-0 bead seeds one classical
    worldline (loadClassicalState, src/pimc.cpp:1006-1029) on the identity
    links, inactive beads unlinked.  Positions are put inside the box
    (Container::putInBC).  Returns (cfg, rng_words or None)."""
    st = parse_state(text)
    nwl = st["num_worldlines"]
    beads = st["beads"]
    m = int(num_slices)
    if beads.shape[0] == m:
        if beads.shape[1] != nwl:
            raise ValueError("state: %d worldlines declared, %d stored" % (nwl, beads.shape[1]))
        pos = beads.copy()
        nxt, prv = st["next"].copy(), st["prev"].copy()
        on = (st["worm_beads"] != 0).astype(np.uint8)
    else:
        t = np.arange(m, dtype=np.int32)[:, None]
        p = np.arange(nwl, dtype=np.int32)[None, :]
        nxt = np.stack(np.broadcast_arrays((t + 1) % m, p), axis=-1).astype(np.int32)
        prv = np.stack(np.broadcast_arrays((t - 1) % m, p), axis=-1).astype(np.int32)
        pos = np.zeros((m, nwl, 3))
        on = np.zeros((m, nwl), dtype=np.uint8)
        k = 0
        for n in range(nwl):
            if st["worm_beads"][0, n]:
                pos[:, k, :] = beads[0, n]
                on[:, k] = 1
                k += 1
        nxt[on == 0] = NO_BEAD
        prv[on == 0] = NO_BEAD
    pos = _put_in_bc(pos, np.broadcast_to(np.asarray(side, dtype=np.float64), (3,)))
    cfg = dict(pos=pos, next=nxt.astype(np.int32), prev=prv.astype(np.int32), on=on,
               worm=np.full(8, -1, dtype=np.int32))
    return cfg, (st["rng"] if restart else None)


# --------------------------------------------------------------------------
# estimator files
# --------------------------------------------------------------------------
def data_name(temperature, tau, pimc_id, num_particles=None, volume=None, side_length=None,
              mu=None, canonical=True):
    """Communicator::init's dataName (src/communicator.cpp:158-170)."""
    if canonical:
        return "%06.3f-%04d-%06.3f-%7.5f-%s" % (temperature, num_particles,
                                                 1.0 * num_particles / volume, tau, pimc_id)
    return "%06.3f-%07.3f-%+08.3f-%7.5f-%s" % (temperature, side_length, mu, tau, pimc_id)


def output_path(out_dir, label, data, canonical=True):
    """File::File naming (src/communicator.cpp:39-46)."""
    return os.path.join(out_dir, "%s-%s-%s.dat" % ("ce" if canonical else "gce", label, data))


def scalar_header(labels):
    """EstimatorBase::initialize's header, "%16s" per label
    (src/estimator.cpp:279-282)."""
    return "".join("%16s" % s for s in labels)


def commented(header):
    """EstimatorBase::prepare replaces the header's first character with '#'
    when it opens a file (src/estimator.cpp:307-309)."""
    return "#" + header[1:] if header else header


ENERGY_LABELS = ("K", "V", "V_ext", "V_int", "E", "E_mu", "K/N", "V/N", "E/N")
VIRIAL_LABELS = ("K_op", "K_cv", "V_op", "V_cv", "E", "E_mu", "K_op/N", "K_cv/N", "V_op/N",
                 "V_cv/N", "E/N", "EEcv*Beta^2", "Ecv*Beta", "dEdB", "CvCov1", "CvCov2",
                 "CvCov3", "E_th", "P")
WIND_MAX = 10                  # SuperfluidFractionEstimator::windMax
NPCFSEP = 50                   # include/common.h:85
MAX_NUM_CYCLES = 40            # PermutationCycleEstimator (estimator.h)


def superfluid_header(wind_max=WIND_MAX):
    """src/estimator.cpp:1975-1978."""
    h = "#%15s%16s%16s%16s" % ("rho_s/rho", "W^2(x)", "W^2(y)", "W^2(z)")
    for w in range(-wind_max, wind_max + 1):
        h += "%16s" % ("P(%+2d)" % w)
    return h + "%16s" % "Area_rho_s"


def pair_correlation_header(side_z, periodic_dims=3):
    """src/estimator.cpp:3187-3195: separations n dR, dR = sqrt(#periodic)
    L_z / (2 NPCFSEP)."""
    dr = 0.5 * np.sqrt(periodic_dims) * side_z / (1.0 * NPCFSEP)
    return "#%15.3E" % 0.0 + "".join("%16.3E" % (n * dr) for n in range(1, NPCFSEP))


def permutation_header(max_cycles=MAX_NUM_CYCLES):
    """src/estimator.cpp:2717-2719."""
    return "#%15d" % 1 + "".join("%16d" % n for n in range(2, max_cycles + 1))


def _dvec_label(v):
    """EstimatorBase::dVecToString (src/estimator.cpp:420-428)."""
    return "(" + ",".join("%+15.8E" % x for x in v) + ")"


def q_header(qvecs):
    """Static structure factor / intermediate scattering function headers
    (src/estimator.cpp:3680-3688, 3782-3790)."""
    q = np.asarray(qvecs, dtype=np.float64).reshape(-1, 3)
    h = "# ESTINF: num_q = %d; " % len(q)
    h += "".join(_dvec_label(v) + " " for v in q)
    h += "\n"
    h += "#%15d" % 0 + "".join("%16d" % n for n in range(1, len(q)))
    return h


def pair_correlation_norm(side, periodic_dims=3):
    """PairCorrelationEstimator's norm (src/estimator.cpp:3214-3222), 3-D."""
    side = np.broadcast_to(np.asarray(side, dtype=np.float64), (3,))
    dr = 0.5 * np.sqrt(periodic_dims) * side[2] / (1.0 * NPCFSEP)
    n = np.arange(NPCFSEP)
    dv = ((n + 1) * dr) ** 3 - (n * dr) ** 3
    return 0.5 * (3.0 / (2.0 * np.pi)) * float(np.prod(side)) / dv


def format_row(values):
    """One bin: "%16.8E" per column (src/estimator.cpp:354-358)."""
    return "".join("%16.8E" % float(v) for v in np.ravel(values))


class EstimatorFile:
    """One estimator output file, opened as Communicator::initFile and
    EstimatorBase::prepare do (src/communicator.cpp:184-192, 226-243;
    src/estimator.cpp:297-321): appended to on a restart, truncated
    otherwise; "# PIMCID: <id>" first when the file is new; the header
    (first character made '#') unless a restart finds the file already
    there.  Scalar estimators that share one file pass their headers
    concatenated and write their columns together on one line."""

    def __init__(self, path, header, pimc_id, restart=False):
        self.path = path
        existed = os.path.exists(path)
        d = os.path.dirname(path)
        if d:
            os.makedirs(d, exist_ok=True)
        self.f = open(path, "a" if restart else "w")
        if not existed:
            self.f.write("# PIMCID: %s\n" % pimc_id)
        if not restart or not existed:
            self.f.write(commented(header) + "\n")
        self.f.flush()

    def output(self, *bins):
        """One line: for each (sums, num_accumulated, norm) in turn,
        sums * norm / num_accumulated as "%16.8E" columns (EstimatorBase::output)."""
        row = ""
        for sums, count, norm in bins:
            vals = np.asarray(sums, dtype=np.float64) * (np.asarray(norm, dtype=np.float64)
                                                        / (1.0 * count))
            row += format_row(vals)
        self.f.write(row + "\n")
        self.f.flush()

    def close(self):
        if self.f:
            self.f.close()
            self.f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Bin:
    """Sums of one estimator's per-sample values over a bin."""

    def __init__(self, ncols):
        self.sums = np.zeros(ncols)
        self.count = 0

    def add(self, values):
        self.sums += np.asarray(values, dtype=np.float64)
        self.count += 1

    def take(self, norm=1.0):
        """(sums, count, norm) for EstimatorFile.output, then reset."""
        out = (self.sums.copy(), self.count, norm)
        self.sums[:] = 0.0
        self.count = 0
        return out


# --------------------------------------------------------------------------
# checkpoints
# --------------------------------------------------------------------------
def save_plain_state(action, cfg, path, move_counts=(), estimator_counts=()):
    """Write the state file of a plain-form run: the device positions with
    the loaded links and active flags, and the MT19937 stream's state.
    The file is written to path + ".bak" and renamed over path, as
    File::reset/rename do (src/communicator.cpp:108-131)."""
    live = dict(cfg)
    live["pos"] = action.positions()
    text = format_state(left_pack(live), action.rng_state(), move_counts, estimator_counts)
    _atomic_write(path, text)
    return text


def resume_plain_state(action, path, num_slices, side):
    """Load a state file into the context and continue its generator."""
    with open(path) as f:
        cfg, rng = load_state(f.read(), num_slices, side, restart=True)
    action.load(cfg)
    if rng is not None:
        action.set_rng_state(rng)
    return cfg


def _atomic_write(path, text):
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    bak = path + ".bak"
    with open(bak, "w") as f:
        f.write(text)
    os.replace(bak, path)


def _walker_rng_words(seed, walker, sweeps):
    """An MTRand::save image for a walker's state file, so that the
    reference can restart from it with its own generator: init_genrand of a
    32-bit seed mixed from (seed, walker, sweeps), left = 0."""
    s = (int(seed) * 0x9E3779B1 + int(walker) * 0x85EBCA77 + int(sweeps) * 0xC2B2AE3D) & 0xFFFFFFFF
    mt = np.zeros(624, dtype=np.uint64)
    mt[0] = s
    for i in range(1, 624):
        prev = int(mt[i - 1])
        mt[i] = (1812433253 * (prev ^ (prev >> 30)) + i) & 0xFFFFFFFF
    return np.concatenate([mt.astype(np.uint32), np.array([0], dtype=np.uint32)])


def save_walkers(walkers, out_dir, seed):
    """Checkpoint every walker: one reference-format state file per walker
    (state, state2, ... as the reference names its paths) with identity
    links, and walkers.json with the sweep counters that index each
    walker's counter-based draws."""
    os.makedirs(out_dir, exist_ok=True)
    allpos = walkers.all_positions()
    sweeps = walkers.sweeps_done()
    stats = walkers.stats_array()
    off = 0
    for w in range(walkers.W):
        n, m = int(walkers.n[w]), int(walkers.m[w])
        pos = allpos[off:off + 3 * n * m].reshape(m, n, 3)
        off += 3 * n * m
        t = np.arange(m, dtype=np.int32)[:, None]
        p = np.arange(n, dtype=np.int32)[None, :]
        cfg = dict(pos=pos,
                   next=np.stack(np.broadcast_arrays((t + 1) % m, p), axis=-1),
                   prev=np.stack(np.broadcast_arrays((t - 1) % m, p), axis=-1),
                   on=np.ones((m, n), dtype=np.uint8))
        st = stats[w]
        moves = [(int(st["accepted"][k]), int(st["attempted"][k])) for k in range(2)]
        text = format_state(cfg, _walker_rng_words(seed, w, int(sweeps[w])), moves,
                            [(int(st["samples"]), int(st["samples"]))])
        _atomic_write(os.path.join(out_dir, "state" if w == 0 else "state%d" % (w + 1)), text)
    meta = dict(seed=int(seed), sweeps=[int(s) for s in sweeps],
                num_ptcl=[int(v) for v in walkers.n], num_slices=[int(v) for v in walkers.m])
    _atomic_write(os.path.join(out_dir, "walkers.json"), json.dumps(meta))


def resume_walkers(walkers, out_dir):
    """Restore the positions and sweep counters written by save_walkers; the
    walkers then continue exactly the chains they would have run."""
    with open(os.path.join(out_dir, "walkers.json")) as f:
        meta = json.load(f)
    if meta["num_ptcl"] != [int(v) for v in walkers.n] or \
            meta["num_slices"] != [int(v) for v in walkers.m]:
        raise ValueError("checkpoint: walker shapes differ from this run's")
    parts = []
    for w in range(walkers.W):
        name = "state" if w == 0 else "state%d" % (w + 1)
        with open(os.path.join(out_dir, name)) as f:
            st = parse_state(f.read())
        parts.append(st["beads"].reshape(-1))
    walkers.set_all_positions(np.concatenate(parts))
    walkers.sync()
    walkers.set_sweeps_done(np.array(meta["sweeps"], dtype=np.uint64))
    return meta
