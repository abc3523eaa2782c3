"""Device-side ERI engine: shells and shell pairs in HBM, class-sorted quartet task lists,
and the launches of the sm_103a class kernels through the C ABI.

Layout in HBM (all owned by torch tensors):
  DeviceShells  per shell: centre[3] f64, l i32, prim_off i32, func_off i32, comp_scale[6] f64;
                per primitive: exponent f64, effective coefficient f64.
  PairSet       per shell pair a 48-byte PairRec (AB, primitive-pair range, shells, Schwarz
                bound); per primitive pair an 80-byte f64 record and a 48-byte f32 record
                (p, 1/2p, P, PA, Kp) -- see csrc/eri_common.cuh.
  tasks         write tasks (24 B: bra, ket, permutation code, output offset) or Fock
                tasks (8 B: bra, ket), grouped by angular-momentum class and sorted by
                primitive-quartet count, largest first (so a launch does not end on its
                longest blocks), equal primitive counts together (a warp's threads run
                the same loop trip counts).
"""
import numpy as np
import torch

from . import _lib
from .basis import COMPONENTS, ShellBasis

PAIR_ORDER = [(0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2)]
PAIR_CLASS = {p: i for i, p in enumerate(PAIR_ORDER)}
NCART = np.array([1, 3, 6, 10])
PAIR_REC, PRIM64, PRIM32, WRITE_TASK = 48, 80, 48, 24
# Primitive pairs with alpha*beta/p |AB|^2 above this (Gaussian-product factor < 1e-24)
# are dropped by the pair builder when screening is on.
PRIM_SCREEN = 55.262
WRITE_TASK_DTYPE = np.dtype([("bra", "<i4"), ("ket", "<i4"), ("code", "<i4"), ("pad", "<i4"),
                             ("off", "<i8")])

# Quartets with many primitive quartets (after the pair screen) of a class that runs one
# thread per quartet run in the split form instead: one warp per quartet, its lanes taking
# the primitive quartets 32 at a time with the same straight-line code, then summing their
# contraction accumulators.  One thread walking them all would make the launch end on a
# few long-running warps.  "Many" is at least HEAVY_PRIM_QUARTETS and twice the class's
# accumulator count (the warp's final sum costs five additions per accumulator).
HEAVY_PRIM_QUARTETS = 32
# Quartets with at least COOP_PRIM_QUARTETS primitive quartets of a class that runs one
# warp per quartet run in the cooperative form: up to eight warps per quartet (as many as
# fit the shared memory), warp w taking primitive quartets w, w + warps, ..., the partial
# sums added in shared memory before one HRR.  The class's time would otherwise have a floor at its heaviest quartet,
# walked by one warp while the other warps of the launch have finished.
COOP_PRIM_QUARTETS = 128
THREAD_FORM, WARP_FORM, GROUPED_FORM, SPLIT_FORM, COOP_FORM, STACKED_FORM = 1, 2, 3, 4, 5, 6
# (class, precision) pairs whose heavy quartets stay on the class's own form (set by the
# autotuner where that measured faster)
SPLIT_OFF = set()


def heavy_threshold(cls):
    """Primitive quartets from which a quartet of class ``cls`` is run in the split form."""
    la, lb, lc, ld = cls
    ne = sum((x + 1) * (x + 2) // 2 for x in range(la, la + lb + 1))
    nf = sum((x + 1) * (x + 2) // 2 for x in range(lc, lc + ld + 1))
    return max(HEAVY_PRIM_QUARTETS, 2 * ne * nf)

_pc_lut = np.full((3, 3), -1, dtype=np.int64)
for _i, (_a, _b) in enumerate(PAIR_ORDER):
    _pc_lut[_a, _b] = _i


def heavy_counts(cls, work_desc):
    """(split, cooperative): how many tasks of a segment whose primitive-quartet counts
    ``work_desc`` are sorted in descending order reach heavy_threshold(cls), and how many
    reach COOP_PRIM_QUARTETS -- both prefixes of the segment."""
    w = -np.asarray(work_desc, dtype=np.int64)
    return (int(np.searchsorted(w, -heavy_threshold(cls), side="right")),
            int(np.searchsorted(w, -COOP_PRIM_QUARTETS, side="right")))


def split_forms(cls, precision, heavy):
    """[(form, first, count)] for a class segment whose tasks are sorted by descending
    primitive-quartet count, with heavy = heavy_counts(cls, ...): the heavy prefix in the
    split form when the class runs one thread per quartet, in the cooperative form when it
    runs one warp per quartet, the rest in the class's form.  form 0 = the class's
    configured form; count None = to the end of the segment."""
    if (cls, precision) in SPLIT_OFF:
        return [(0, 0, None)]
    form = _lib.lib().gs_class_form(*cls, precision)
    if form == THREAD_FORM:
        h, hform = heavy[0], SPLIT_FORM
    elif form in (WARP_FORM, GROUPED_FORM, STACKED_FORM):
        h, hform = heavy[1], COOP_FORM
    else:
        h, hform = 0, 0
    if h <= 0:
        return [(0, 0, None)]
    return [(hform, 0, h), (form, h, None)]


def mixed_prefix(cls, heavy, mixed_cut):
    """The heavy prefix of a class segment in a mixed-precision build, whose partitioned
    launch (gs_fock_jk_mixed) evaluates every quartet in the class's configured form.
    Returns (h, [(precision, form, first, count, prec_lo, prec_hi)]): tasks [0, h) run as
    banded launches -- FP64 for density-weighted bounds at or above ``mixed_cut``, FP32
    below, the same bands as the partition -- each precision's heavy tasks in its heavy
    form (split_forms) and the rest of the prefix in its configured form; the partitioned
    launch takes [h, end).  (0, []) when neither precision has a heavy form here."""
    parts = {p: split_forms(cls, p, heavy) for p in (64, 32)}
    h = max((pp[0][2] for pp in parts.values() if len(pp) > 1), default=0)
    if h == 0:
        return 0, []
    out = []
    for p, lo, hi in ((64, mixed_cut, float("inf")), (32, 0.0, mixed_cut)):
        pp = parts[p]
        c = pp[0][2] if len(pp) > 1 else 0
        if c > 0:
            out.append((p, pp[0][0], 0, c, lo, hi))
        if c < h:
            out.append((p, 0, c, h - c, lo, hi))
    return h, out


_SIDE = {}


class HeavyLane:
    """Side streams of a build, forked from the caller's stream before their first launch
    and joined back by ``join``.  Side 0 takes the heavy prefixes of the classes: their few
    long blocks then run beside the class launches instead of leaving most SMs idle while
    they finish.  Side 1 takes every other class's launch of a plain (unpartitioned)
    build, so that one class's last partial wave overlaps the next class's first."""

    def __init__(self, device, stream=None):
        d = indexed_device(device)
        self.main = stream or torch.cuda.current_stream(d)
        if d not in _SIDE:
            _SIDE[d] = (torch.cuda.Stream(device=d), torch.cuda.Stream(device=d))
        self.sides = _SIDE[d]
        self.forked = [False, False]

    def stream(self, k=0):
        """Side stream k (as the C ABI takes it), forked on first use."""
        if not self.forked[k]:
            self.sides[k].wait_stream(self.main)
            self.forked[k] = True
        return _lib.stream(self.sides[k])

    def alternate(self, i):
        """The stream of the i-th class launch of a plain build: the caller's or side 1."""
        return _lib.stream(self.main) if i % 2 == 0 else self.stream(1)

    def join(self):
        for k in (0, 1):
            if self.forked[k]:
                self.main.wait_stream(self.sides[k])
                self.forked[k] = False


def check_record_sizes(lib=None):
    """The library's pair, primitive-pair and task record sizes (``gs_record_sizes``, a host
    call) must equal the layouts this module packs; raises GsError on a mismatch."""
    sizes = np.zeros(4, dtype=np.int32)
    _lib.check((lib or _lib.lib()).gs_record_sizes(sizes.ctypes.data), "gs_record_sizes")
    if tuple(int(x) for x in sizes) != (PAIR_REC, PRIM64, PRIM32, WRITE_TASK):
        raise _lib.GsError(f"record sizes mismatch: library {tuple(sizes)}, host "
                           f"{(PAIR_REC, PRIM64, PRIM32, WRITE_TASK)}")


def indexed_device(device):
    """The device with its index made explicit ('cuda' -> 'cuda:<current>'), so that a
    comparison with a tensor's device is exact."""
    d = torch.device(device)
    if d.type == "cuda" and d.index is None:
        d = torch.device("cuda", torch.cuda.current_device())
    return d


def _check_device_tensor(t, device, what, shape=None):
    """Tensors handed to a kernel must be float64 on the engine's CUDA device (a host
    pointer or a float32 buffer would be read as the wrong memory, a tensor on another
    GPU as another device's memory)."""
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64:
        raise _lib.GsError(f"{what} must be a float64 CUDA tensor")
    if t.device != indexed_device(device):
        raise _lib.GsError(f"{what} is on {t.device}, the engine on {indexed_device(device)}")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{what} has shape {tuple(t.shape)}, expected {tuple(shape)}")
    if shape is None and not t.is_contiguous():
        raise ValueError(f"{what} must be contiguous")


class DeviceShells:
    """A ShellBasis copied to the device."""

    def __init__(self, sb: ShellBasis, device="cuda"):
        self.host = sb
        self.device = indexed_device(device)

        def t(a, dt):
            return torch.as_tensor(np.ascontiguousarray(a), dtype=dt).to(self.device)

        self.centre = t(sb.centre, torch.float64)
        self.l = t(sb.l, torch.int32)
        self.prim_off = t(sb.prim_off, torch.int32)
        self.expo = t(sb.expo, torch.float64)
        self.coef = t(sb.coef, torch.float64)
        self.comp_scale = t(sb.comp_scale, torch.float64)
        self.func_off = t(sb.func_off, torch.int32)
        self.nprim = t(sb.nprim, torch.int64)          # primitives per shell (device planning)
        self.nshell = sb.nshell
        self.nbf = sb.nbf


def pair_groups(sizes, lanes=32):
    """Start indices (and the end) of groups of consecutive shell pairs whose primitive
    pairs total at most ``lanes``: aligned runs of four pairs when they fit, else of two,
    else single pairs (vectorised; a pair with more primitive pairs is a group of its own)."""
    sizes = np.asarray(sizes, dtype=np.int64)
    n = len(sizes)
    if n == 0:
        return np.zeros(1, dtype=np.int32)
    m = -(-n // 4) * 4
    sz = np.zeros(m, dtype=np.int64)
    sz[:n] = sizes
    quad = np.repeat(sz.reshape(-1, 4).sum(1) <= lanes, 4)
    half = np.repeat(sz.reshape(-1, 2).sum(1) <= lanes, 2)
    r = np.tile(np.arange(4), m // 4)
    start = (r == 0) | ((r == 2) & ~quad) | ((r & 1).astype(bool) & ~quad & ~half)
    out = np.flatnonzero(start[:n]).astype(np.int32)
    return np.concatenate([out, np.array([n], dtype=np.int32)])


def pair_groups_device(sizes, lanes=32):
    """pair_groups on a device tensor of sizes (the same groups; int32 device tensor)."""
    dev = sizes.device
    n = sizes.numel()
    if n == 0:
        return torch.zeros(1, dtype=torch.int32, device=dev)
    m = -(-n // 4) * 4
    sz = torch.zeros(m, dtype=torch.int64, device=dev)
    sz[:n] = sizes
    quad = (sz.view(-1, 4).sum(1) <= lanes).repeat_interleave(4)
    half = (sz.view(-1, 2).sum(1) <= lanes).repeat_interleave(2)
    r = torch.arange(m, device=dev) % 4
    start = (r == 0) | ((r == 2) & ~quad) | (((r & 1) == 1) & ~quad & ~half)
    out = torch.nonzero(start[:n]).flatten().to(torch.int32)
    return torch.cat([out, torch.tensor([n], dtype=torch.int32, device=dev)])


def check_shell_indices(idx, nshell, what):
    """Shell indices handed to the kernels must lie in [0, nshell): a kernel trusts them."""
    idx = np.asarray(idx)
    if idx.size and (int(idx.min()) < 0 or int(idx.max()) >= nshell):
        raise ValueError(f"{what} hold a shell index outside [0, {nshell})")


class PairSet:
    """Shell pairs (la >= lb inside each pair) with their primitive-pair records."""

    def __init__(self, ds: DeviceShells, pair_shells, want32=True, stream=None, max_exp=0.0):
        ps = np.ascontiguousarray(pair_shells, dtype=np.int32).reshape(-1, 2)
        sb = ds.host
        check_shell_indices(ps, sb.nshell, "shell pairs")
        if len(ps) and np.any(sb.l[ps[:, 0]] < sb.l[ps[:, 1]]):
            raise ValueError("pair shells must have l[first] >= l[second]")
        npp = sb.nprim[ps[:, 0]].astype(np.int64) * sb.nprim[ps[:, 1]]
        off = np.zeros(len(ps) + 1, dtype=np.int64)
        off[1:] = np.cumsum(npp)
        if off[-1] >= 2 ** 31:
            raise ValueError("too many primitive pairs for one PairSet")
        self.ds = ds
        self.n = len(ps)
        self.host_shells = ps
        self.nprim = npp
        self.la = sb.l[ps[:, 0]] if len(ps) else np.zeros(0, np.int32)
        self.lb = sb.l[ps[:, 1]] if len(ps) else np.zeros(0, np.int32)
        dev = ds.device
        self.shells = torch.as_tensor(ps).to(dev)
        self.prim_start = torch.as_tensor(off[:-1].astype(np.int32)).to(dev)
        self.rec = torch.empty(max(1, self.n) * PAIR_REC, dtype=torch.uint8, device=dev)
        total = max(1, int(off[-1]))
        self.p64 = torch.empty(total * PRIM64, dtype=torch.uint8, device=dev)
        self.p32 = torch.empty(total * PRIM32, dtype=torch.uint8, device=dev) if want32 else None
        self.nprim_pairs = int(off[-1])
        self.max_exp = max_exp
        # consecutive pairs packed into warps of at most 32 primitive pairs (the pair build)
        self.groups = torch.as_tensor(pair_groups(npp)).to(dev)
        self.ngroups = int(self.groups.numel()) - 1
        self.kept = torch.zeros(max(1, self.n), dtype=torch.int32, device=dev)
        self.build(stream)
        # primitive pairs kept per shell pair (the work per pair after screening)
        self.nprim = self.kept[:self.n].cpu().numpy().astype(np.int64)

    def build(self, stream=None, want32=True):
        """(Re)compute the pair records (kernel K0) from the device shells; with
        ``want32=False`` only the FP64 records (enough for FP64-only evaluation)."""
        ds = self.ds
        L = _lib.lib()
        p32 = self.p32 if want32 else None
        _lib.check(L.gs_pairs_build(_lib.ptr(ds.centre), _lib.ptr(ds.l), _lib.ptr(ds.prim_off),
                                    _lib.ptr(ds.expo), _lib.ptr(ds.coef), self.n,
                                    _lib.ptr(self.shells), _lib.ptr(self.prim_start),
                                    _lib.ptr(self.rec), _lib.ptr(self.p64), _lib.ptr(p32),
                                    float(self.max_exp), _lib.ptr(self.kept), self.ngroups,
                                    _lib.ptr(self.groups), _lib.stream(stream)), "gs_pairs_build")

    def prims(self, precision):
        return self.p64 if precision == 64 else self.p32


class DevicePairSet(PairSet):
    """A PairSet planned on the device from a device tensor of shell pairs (m, 2) int32,
    l[first] >= l[second] (as canonical quartets give them): the same records, groups and
    kept counts; the host copies of the pair list and counts are made when first read."""

    def __init__(self, ds: DeviceShells, pair_shells, want32=True, stream=None, max_exp=0.0):
        dev = ds.device
        ps = pair_shells.to(device=dev, dtype=torch.int32).reshape(-1, 2).contiguous()
        m = ps.shape[0]
        npp = ds.nprim[ps[:, 0].long()] * ds.nprim[ps[:, 1].long()]
        off = torch.cumsum(npp, 0)
        total = int(off[-1]) if m else 0
        if total >= 2 ** 31:
            raise ValueError("too many primitive pairs for one PairSet")
        self.ds = ds
        self.n = m
        self.shells = ps
        self.prim_start = (off - npp).to(torch.int32)
        self.rec = torch.empty(max(1, m) * PAIR_REC, dtype=torch.uint8, device=dev)
        t = max(1, total)
        self.p64 = torch.empty(t * PRIM64, dtype=torch.uint8, device=dev)
        self.p32 = torch.empty(t * PRIM32, dtype=torch.uint8, device=dev) if want32 else None
        self.nprim_pairs = total
        self.max_exp = max_exp
        self.groups = pair_groups_device(npp, 32)
        self.ngroups = int(self.groups.numel()) - 1
        self.kept = torch.zeros(max(1, m), dtype=torch.int32, device=dev)
        self.build(stream)
        self.nprim_dev = self.kept[:m].long()

    def __getattr__(self, name):
        # host copies, made on first use
        if name == "host_shells":
            v = self.shells.cpu().numpy()
        elif name == "nprim":
            v = self.nprim_dev.cpu().numpy()
        elif name in ("la", "lb"):
            k = 0 if name == "la" else 1
            v = self.ds.host.l[self.shells[:, k].cpu().numpy()]
        else:
            raise AttributeError(name)
        setattr(self, name, v)
        return v


_DEVICE_LUTS = {}


def _device_luts(dev):
    """The canonicalisation and block-size tables (and each pair-class combination's
    heavy threshold) on a device."""
    if dev not in _DEVICE_LUTS:
        pos, code, pcb, pck = _CANON_LUT
        thr = [heavy_threshold(PAIR_ORDER[c // 6] + PAIR_ORDER[c % 6]) for c in range(36)]
        _DEVICE_LUTS[dev] = {
            "pos": torch.as_tensor(np.asarray(pos, dtype=np.int64)).to(dev),
            "code": torch.as_tensor(np.asarray(code, dtype=np.int32)).to(dev),
            "cls": torch.as_tensor(np.asarray(pcb * 6 + pck, dtype=np.int64)).to(dev),
            "size": torch.as_tensor(np.asarray(_SIZE_LUT, dtype=np.int64)).to(dev),
            "thr": torch.as_tensor(np.asarray(thr, dtype=np.int64)).to(dev),
        }
    return _DEVICE_LUTS[dev]


# ---------------------------------------------------------------------- shell-quartet blocks
def _canonicalize_rows(l4):
    """canonicalize, evaluated row by row from the rule (the table below is built from it)."""
    la, lb, lc, ld = l4[:, 0], l4[:, 1], l4[:, 2], l4[:, 3]
    s_ab = la < lb
    s_cd = lc < ld
    A = np.where(s_ab, 1, 0); B = 1 - A
    C = np.where(s_cd, 3, 2); Dd = 5 - C
    pc1 = _pc_lut[np.maximum(la, lb), np.minimum(la, lb)]
    pc2 = _pc_lut[np.maximum(lc, ld), np.minimum(lc, ld)]
    s_bk = pc2 > pc1
    code = np.where(s_bk, s_cd.astype(np.int32) | (s_ab.astype(np.int32) << 1) | 4,
                    s_ab.astype(np.int32) | (s_cd.astype(np.int32) << 1))
    pos = np.stack([np.where(s_bk, C, A), np.where(s_bk, Dd, B),
                    np.where(s_bk, A, C), np.where(s_bk, B, Dd)], axis=1)
    return pos, code.astype(np.int32), np.where(s_bk, pc2, pc1), np.where(s_bk, pc1, pc2)


# canonicalize's results and the block size for each of the 81 (la, lb, lc, ld) with l <= 2,
# indexed by ((la*3 + lb)*3 + lc)*3 + ld: a gather per quartet instead of a dozen
# elementwise passes over the batch
_L4_ALL = np.array([[a, b, c, d] for a in range(3) for b in range(3) for c in range(3)
                    for d in range(3)], dtype=np.int64)
_CANON_LUT = _canonicalize_rows(_L4_ALL)
_SIZE_LUT = np.prod(NCART[_L4_ALL], axis=1)


def _l4_index(l4):
    l4 = np.asarray(l4, dtype=np.int64)
    return ((l4[:, 0] * 3 + l4[:, 1]) * 3 + l4[:, 2]) * 3 + l4[:, 3]


def canonicalize(l4):
    """Per quartet of angular momenta (n,4): canonical order (bra pair class >= ket pair
    class, la >= lb, lc >= ld), the 3-bit permutation code, and index maps."""
    i = _l4_index(l4)
    pos, code, pcb, pck = _CANON_LUT
    return pos[i], code[i], pcb[i], pck[i]


class QuartetBatch:
    """A batch of shell quartets (n,4 shell indices, any order) evaluated into one flat f64
    buffer: quartet q's block occupies out[off[q] : off[q] + na*nb*nc*nd] in the caller's
    (a,b,c,d) order, row-major.  Host preparation sorts the quartets by class and
    primitive counts; ``run`` launches one kernel per class."""

    def __init__(self, ds: DeviceShells, quartets, want32=True, max_exp=0.0, plan="host"):
        """``plan="device"``: the same planning with torch on the device (quartets may be a
        host array or a device tensor); only the class histogram and heavy counts come back
        to the host, and the host copies of offsets and primitive counts are made when
        first read."""
        if plan == "device":
            self._plan_device(ds, quartets, want32, max_exp)
            return
        if plan != "host":
            raise ValueError(f"plan must be 'host' or 'device', not {plan!r}")
        q = np.ascontiguousarray(quartets, dtype=np.int64).reshape(-1, 4)
        sb = ds.host
        check_shell_indices(q, sb.nshell, "shell quartets")
        n = len(q)
        l4 = sb.l[q]
        li = _l4_index(l4)
        pos, code, pcb, pck = (x[li] for x in _CANON_LUT)
        qc = np.take_along_axis(q, pos, axis=1)          # canonical shells
        size = _SIZE_LUT[li]
        off = np.zeros(n + 1, dtype=np.int64)
        off[1:] = np.cumsum(size)
        self.n = n
        self.offsets = off
        self.total = int(off[-1])
        pairs = np.concatenate([qc[:, 0:2], qc[:, 2:4]], axis=0)
        self.pairs = PairSet(ds, pairs, want32=want32, max_exp=max_exp)
        self.full_prim_quartets = int(np.sum(sb.nprim[qc[:, 0]].astype(np.int64) * sb.nprim[qc[:, 1]] *
                                             sb.nprim[qc[:, 2]] * sb.nprim[qc[:, 3]]))
        nb = self.pairs.nprim[:n]
        nk = self.pairs.nprim[n:]
        cls = pcb * 6 + pck
        # within a class, most primitive quartets first (the longest blocks start first, so
        # the short ones fill the end of the launch), equal (K_bra, K_ket) kept together so
        # that the lanes of a warp run the same loop trip counts: one packed key (class,
        # then descending nb*nk, nb, nk) and a stable sort, the order of a lexsort on the four
        wb = int(nb.max()).bit_length() if n else 1
        wk = int(nk.max()).bit_length() if n else 1
        ww = int((nb * nk).max()).bit_length() if n else 1
        key = cls.astype(np.int64)
        key = (key << ww) | ((1 << ww) - 1 - nb * nk)
        key = (key << wb) | ((1 << wb) - 1 - nb)
        key = (key << wk) | ((1 << wk) - 1 - nk)
        wi = int(n).bit_length()
        if 6 + ww + wb + wk + wi <= 62:
            # the index as the last key field makes every key distinct: a plain value sort
            # gives the stable order (and is faster than a stable argsort)
            order = np.sort((key << wi) | np.arange(n, dtype=np.int64)) & ((1 << wi) - 1)
        else:
            order = np.argsort(key, kind="stable")
        tasks = np.zeros(n, dtype=WRITE_TASK_DTYPE)
        tasks["bra"] = order
        tasks["ket"] = order + n
        tasks["code"] = code[order]
        tasks["off"] = off[:-1][order]
        self.prim_quartets = int(np.sum(nb * nk))
        scls = cls[order]
        self.segments = []
        starts = np.flatnonzero(np.diff(np.concatenate([[-1], scls]))) if n else []
        bounds = list(starts) + [n]
        for s, e in zip(bounds[:-1], bounds[1:]):
            c = int(scls[s])
            (la, lb), (lc, ld) = PAIR_ORDER[c // 6], PAIR_ORDER[c % 6]
            self.segments.append(((la, lb, lc, ld), int(s), int(e)))
        self.tasks_host = tasks
        self.tasks = torch.as_tensor(tasks.view(np.uint8)).to(ds.device)
        self.ds = ds
        self.sorted_bra_nprim = nb[order]
        self.sorted_ket_nprim = nk[order]
        work = self.sorted_bra_nprim * self.sorted_ket_nprim
        self.heavy = [heavy_counts(cls, work[s:e]) for cls, s, e in self.segments]

    def _plan_device(self, ds, quartets, want32, max_exp):
        dev = ds.device
        sb = ds.host
        q = torch.as_tensor(quartets).to(device=dev, dtype=torch.int64).reshape(-1, 4)
        n = q.shape[0]
        if n and (int(q.min()) < 0 or int(q.max()) >= sb.nshell):
            raise ValueError(f"shell quartets hold a shell index outside [0, {sb.nshell})")
        lut = _device_luts(dev)
        l4 = ds.l.long()[q]
        li = ((l4[:, 0] * 3 + l4[:, 1]) * 3 + l4[:, 2]) * 3 + l4[:, 3]
        qc = torch.gather(q, 1, lut["pos"][li])             # canonical shells
        off = torch.zeros(n + 1, dtype=torch.int64, device=dev)
        off[1:] = torch.cumsum(lut["size"][li], 0)
        self.n = n
        self._offsets_dev = off
        self.total = int(off[-1])
        self.pairs = DevicePairSet(ds, torch.cat([qc[:, 0:2], qc[:, 2:4]], 0), want32=want32,
                                   max_exp=max_exp)
        npr = ds.nprim
        self.full_prim_quartets = int((npr[qc[:, 0]] * npr[qc[:, 1]] * npr[qc[:, 2]] *
                                       npr[qc[:, 3]]).sum()) if n else 0
        nb = self.pairs.nprim_dev[:n]
        nk = self.pairs.nprim_dev[n:]
        w = nb * nk
        cls = lut["cls"][li]
        self.prim_quartets = int(w.sum()) if n else 0
        # the host form's order: class, then descending nb*nk, nb, nk; ties in input order
        wb = int(nb.max()).bit_length() if n else 1
        wk = int(nk.max()).bit_length() if n else 1
        ww = int(w.max()).bit_length() if n else 1
        key = (cls << ww) | ((1 << ww) - 1 - w)
        key = (key << wb) | ((1 << wb) - 1 - nb)
        key = (key << wk) | ((1 << wk) - 1 - nk)
        order = torch.sort(key, stable=True).indices
        tasks = torch.zeros((n, 6), dtype=torch.int32, device=dev)   # WRITE_TASK layout
        tasks[:, 0] = order.to(torch.int32)
        tasks[:, 1] = (order + n).to(torch.int32)
        tasks[:, 2] = lut["code"][li][order]
        tasks[:, 4:6] = off[:-1][order].contiguous().view(torch.int32).view(n, 2)
        self.tasks = tasks.view(torch.uint8).reshape(-1)
        self.ds = ds
        scls = cls[order]
        ws = w[order]
        nper = torch.bincount(scls, minlength=36).cpu().numpy()
        hs = torch.zeros(36, dtype=torch.int64, device=dev).index_add_(
            0, scls, (ws >= lut["thr"][scls]).long())
        hc = torch.zeros(36, dtype=torch.int64, device=dev).index_add_(
            0, scls, (ws >= COOP_PRIM_QUARTETS).long())
        hs, hc = hs.cpu().numpy(), hc.cpu().numpy()
        self.segments, self.heavy = [], []
        start = 0
        for c in range(36):
            if nper[c]:
                (la, lb), (lc, ld) = PAIR_ORDER[c // 6], PAIR_ORDER[c % 6]
                self.segments.append(((la, lb, lc, ld), start, start + int(nper[c])))
                self.heavy.append((int(hs[c]), int(hc[c])))
                start += int(nper[c])
        self._sorted_dev = (nb[order], nk[order])

    def __getattr__(self, name):
        # host copies of a device-planned batch, made on first use
        if name == "offsets" and "_offsets_dev" in self.__dict__:
            v = self._offsets_dev.cpu().numpy()
        elif name in ("sorted_bra_nprim", "sorted_ket_nprim") and "_sorted_dev" in self.__dict__:
            v = self._sorted_dev[0 if name == "sorted_bra_nprim" else 1].cpu().numpy()
        elif name == "tasks_host" and "_sorted_dev" in self.__dict__:
            v = self.tasks.cpu().numpy().view(WRITE_TASK_DTYPE)
        else:
            raise AttributeError(name)
        setattr(self, name, v)
        return v

    def class_counts(self):
        return {cls: e - s for cls, s, e in self.segments}

    def launch_count(self, precision=64):
        """Kernel launches one ``run`` makes with the current kernel forms: one per class,
        and one more for a class whose heavy prefix runs in its own form."""
        n = 0
        for (cls, s, e), heavy in zip(self.segments, self.heavy):
            for form, first, count in split_forms(cls, precision, heavy):
                n += ((e - s - first) if count is None else count) > 0
        return n

    def run(self, out, precision=64, stream=None, classes=None):
        _check_device_tensor(out, self.ds.device, "output buffer")
        if out.numel() < self.total:
            raise ValueError(f"output buffer holds {out.numel()} doubles, the blocks need {self.total}")
        L = _lib.lib()
        st = _lib.stream(stream)
        lane = HeavyLane(self.ds.device, stream)
        base = self.tasks.data_ptr()
        prims = self.pairs.prims(precision)
        plan = [(cls, s, e, split_forms(cls, precision, heavy))
                for (cls, s, e), heavy in zip(self.segments, self.heavy)
                if classes is None or cls in classes]
        # heavy prefixes first, on side 0; then every class's rest, alternating streams
        for heavy_pass in (True, False):
            for i, (cls, s, e, parts) in enumerate(plan):
                for k, (form, first, count) in enumerate(parts):
                    if (k == 0 and len(parts) > 1) != heavy_pass:
                        continue
                    n = (e - s - first) if count is None else count
                    rc = L.gs_eri_blocks(*cls, precision | (form << 8), _lib.ptr(self.pairs.rec),
                                         _lib.ptr(prims), _lib.ptr(self.ds.comp_scale), n,
                                         base + (s + first) * WRITE_TASK, _lib.ptr(out),
                                         lane.stream() if heavy_pass else lane.alternate(i))
                    _lib.check(rc, f"gs_eri_blocks{cls}")
        lane.join()
        return out


def eri_blocks(sb: ShellBasis, quartets, precision=64, device="cuda"):
    """Convenience: blocks of the given shell quartets, returned as a host f64 array."""
    ds = DeviceShells(sb, device)
    batch = QuartetBatch(ds, quartets, want32=precision == 32)
    out = torch.zeros(max(1, batch.total), dtype=torch.float64, device=ds.device)
    batch.run(out, precision)
    return out[:batch.total].cpu().numpy(), batch.offsets


# ---------------------------------------------------------------------- Fock (J/K) engine
class JKEngine:
    """Integral-direct Coulomb/exchange builder over all unique shell quartets of one
    basis, with Schwarz screening (task list built once per geometry) and optional
    density-weighted screening / precision selection per call."""

    def __init__(self, sb: ShellBasis, device="cuda", schwarz_thr=1e-12, want32=True,
                 max_exp=PRIM_SCREEN):
        self.sb = sb
        self.ds = ds = DeviceShells(sb, device)
        self.dev = ds.device
        ns = sb.nshell
        i, j = np.tril_indices(ns)                      # shell i >= shell j
        swap = sb.l[i] < sb.l[j]
        sa = np.where(swap, j, i)
        sbb = np.where(swap, i, j)
        self.pairs = PairSet(ds, np.stack([sa, sbb], axis=1), want32=want32, max_exp=max_exp)
        self.pair_class = _pc_lut[sb.l[sa], sb.l[sbb]]
        self.npairs = len(sa)
        self.schwarz_thr = schwarz_thr
        self.q = torch.zeros(self.npairs, dtype=torch.float64, device=self.dev)
        L = _lib.lib()
        for c, (la, lb) in enumerate(PAIR_ORDER):
            idx = np.flatnonzero(self.pair_class == c).astype(np.int32)
            if len(idx) == 0:
                continue
            it = torch.as_tensor(idx).to(self.dev)
            _lib.check(L.gs_schwarz(la, lb, _lib.ptr(self.pairs.rec), _lib.ptr(self.pairs.p64),
                                    _lib.ptr(ds.comp_scale), len(idx), _lib.ptr(it),
                                    _lib.ptr(self.q), self.npairs, _lib.stream()), "gs_schwarz")
        self._build_tasks()
        # function -> shell map for per-shell-block density maxima
        self.func_shell = torch.as_tensor(np.repeat(np.arange(ns), sb.nfunc)).to(self.dev)

    def _build_tasks(self):
        dev = self.dev
        q = self.q
        nprim = torch.as_tensor(self.pairs.nprim).to(dev)
        self.segments = []
        self.heavy = []           # heavy_counts of each segment
        chunks = []
        ntot = 0
        thr = self.schwarz_thr
        pc = torch.as_tensor(self.pair_class).to(dev)
        for cb in range(len(PAIR_ORDER)):
            bra_ids = torch.nonzero(pc == cb).flatten()
            if bra_ids.numel() == 0:
                continue
            qb, ob = torch.sort(q[bra_ids], descending=True)
            bra_sorted = bra_ids[ob]
            for ck in range(cb + 1):
                ket_ids = torch.nonzero(pc == ck).flatten()
                if ket_ids.numel() == 0:
                    continue
                qk, ok = torch.sort(q[ket_ids], descending=True)
                ket_sorted = ket_ids[ok]
                # number of kets with qb*qk >= thr: prefix of the descending list
                need = torch.where(qb > 0, thr / qb, torch.full_like(qb, float("inf")))
                cnt = torch.searchsorted(-qk.contiguous(), -need.contiguous(), right=True)
                if cb == ck:
                    start = torch.arange(len(qb), device=dev)
                    cnt = torch.clamp(cnt - start, min=0)
                else:
                    start = torch.zeros(len(qb), dtype=torch.int64, device=dev)
                total = int(cnt.sum())
                if total == 0:
                    continue
                bra_pos = torch.repeat_interleave(torch.arange(len(qb), device=dev), cnt)
                first = torch.cumsum(cnt, 0) - cnt
                within = torch.arange(total, device=dev) - first[bra_pos]
                ket_pos = start[bra_pos] + within
                bra = bra_sorted[bra_pos]
                ket = ket_sorted[ket_pos]
                # most primitive quartets first (longest tasks start first), equal
                # (K_bra, K_ket) together
                key = (nprim[bra] * nprim[ket]) * 4096 + nprim[bra] * 64 + nprim[ket]
                key, o = torch.sort(key, descending=True, stable=True)
                t = torch.stack([bra[o], ket[o]], dim=1).to(torch.int32)
                (la, lb), (lc, ld) = PAIR_ORDER[cb], PAIR_ORDER[ck]
                self.segments.append(((la, lb, lc, ld), ntot, ntot + total))
                self.heavy.append((int((key >= heavy_threshold((la, lb, lc, ld)) * 4096).sum()),
                                   int((key >= COOP_PRIM_QUARTETS * 4096).sum())))
                chunks.append(t)
                ntot += total
        self.tasks = torch.cat(chunks, 0).contiguous() if chunks else \
            torch.zeros((1, 2), dtype=torch.int32, device=dev)
        self.ntasks = ntot

    def shell_dmax(self, mats):
        """max |P_ij| over each (shell, shell) block, over all given matrices."""
        ns = self.sb.nshell
        m = torch.stack([x.abs() for x in mats]).amax(0)
        fs = self.func_shell
        rows = torch.full((ns, m.shape[1]), 0.0, dtype=torch.float64, device=self.dev)
        rows.index_reduce_(0, fs, m, "amax", include_self=True)
        out = torch.full((ns, ns), 0.0, dtype=torch.float64, device=self.dev)
        out.index_reduce_(1, fs, rows, "amax", include_self=True)
        return out.contiguous()

    def jk(self, pj=None, pk=(), precision=64, screen_thr=0.0, mixed_cut=None, stream=None,
           classes=None):
        """J[pj] and K[pk_s] (symmetric densities, nbf x nbf f64 device tensors).

        precision 64 or 32 evaluates every task in that precision.  With ``mixed_cut``
        the quartets whose density-weighted bound is below it run in f32 and the rest in
        f64 (accumulation is always f64).  ``screen_thr`` > 0 additionally skips quartets
        whose density-weighted bound is below it."""
        n = self.sb.nbf
        dev = self.dev
        pk = list(pk)
        nk = len(pk)
        for d in ([pj] if pj is not None else []) + pk:
            _check_device_tensor(d, dev, "density matrix", (n, n))
        jbuf = torch.zeros((n, n), dtype=torch.float64, device=dev) if pj is not None else None
        kbuf = torch.zeros((max(nk, 1), n, n), dtype=torch.float64, device=dev) if nk else None
        pj_c = pj.contiguous() if pj is not None else None
        pk_c = torch.stack(pk).contiguous() if nk else None
        dmax = None
        runs = [(precision, 0.0, float("inf"))]
        if mixed_cut is not None or screen_thr > 0:
            mats = ([pj] if pj is not None else []) + pk
            dmax = self.shell_dmax(mats)
            thr = screen_thr if screen_thr > 0 else 1e-300
            if mixed_cut is not None:
                runs = [(64, mixed_cut, float("inf")), (32, 0.0, mixed_cut)]
            else:
                runs = [(precision, 0.0, float("inf"))]
        else:
            thr = 0.0
        L = _lib.lib()
        st = _lib.stream(stream)
        lane = HeavyLane(dev, stream)
        base = self.tasks.data_ptr()
        if mixed_cut is not None:
            need = max(L.gs_fock_jk_mixed_workspace(e - s) for _, s, e in self.segments)
            if getattr(self, "_ws", None) is None or self._ws.numel() < need:
                self._ws = torch.empty(int(need), dtype=torch.uint8, device=dev)
            for (cls, s, e), heavy in zip(self.segments, self.heavy):
                if classes is not None and cls not in classes:
                    continue
                # the heavy prefix in the heavy forms: banded launches per precision (the
                # same density-weighted bound and cut as the partition)
                h, launches = mixed_prefix(cls, heavy, mixed_cut)
                for prec, form, first, count, lo, hi in launches:
                    rc = L.gs_fock_jk(*cls, prec | (form << 8), _lib.ptr(self.pairs.rec),
                                      _lib.ptr(self.pairs.prims(prec)),
                                      _lib.ptr(self.ds.comp_scale), _lib.ptr(self.ds.func_off),
                                      self.sb.nshell, n, count, base + (s + first) * 8,
                                      _lib.ptr(pj_c), _lib.ptr(jbuf), nk, _lib.ptr(pk_c),
                                      _lib.ptr(kbuf), _lib.ptr(dmax), thr, lo, hi, lane.stream())
                    _lib.check(rc, f"gs_fock_jk{cls}")
                rc = L.gs_fock_jk_mixed(*cls, _lib.ptr(self.pairs.rec), _lib.ptr(self.pairs.p64),
                                        _lib.ptr(self.pairs.p32), _lib.ptr(self.ds.comp_scale),
                                        _lib.ptr(self.ds.func_off), self.sb.nshell, n, e - s - h,
                                        base + (s + h) * 8, _lib.ptr(pj_c), _lib.ptr(jbuf), nk,
                                        _lib.ptr(pk_c), _lib.ptr(kbuf), _lib.ptr(dmax), thr,
                                        mixed_cut, _lib.ptr(self._ws), self._ws.numel(), st)
                _lib.check(rc, f"gs_fock_jk_mixed{cls}")
            runs = []
        for prec, lo, hi in runs:
            prims = self.pairs.prims(prec)
            plan = [(cls, s, e, split_forms(cls, prec, heavy))
                    for (cls, s, e), heavy in zip(self.segments, self.heavy)
                    if classes is None or cls in classes]
            # heavy prefixes first, on side 0; then every class's rest, alternating streams
            for heavy_pass in (True, False):
                for i, (cls, s, e, parts) in enumerate(plan):
                    for k, (form, first, count) in enumerate(parts):
                        if (k == 0 and len(parts) > 1) != heavy_pass:
                            continue
                        m = (e - s - first) if count is None else count
                        rc = L.gs_fock_jk(*cls, prec | (form << 8), _lib.ptr(self.pairs.rec),
                                          _lib.ptr(prims), _lib.ptr(self.ds.comp_scale),
                                          _lib.ptr(self.ds.func_off), self.sb.nshell, n, m,
                                          base + (s + first) * 8, _lib.ptr(pj_c), _lib.ptr(jbuf),
                                          nk, _lib.ptr(pk_c), _lib.ptr(kbuf), _lib.ptr(dmax), thr,
                                          lo, hi, lane.stream() if heavy_pass else lane.alternate(i))
                        _lib.check(rc, f"gs_fock_jk{cls}")
        lane.join()
        J = (jbuf + jbuf.T) if jbuf is not None else None
        K = [kbuf[s] + kbuf[s].T for s in range(nk)]
        return J, K
