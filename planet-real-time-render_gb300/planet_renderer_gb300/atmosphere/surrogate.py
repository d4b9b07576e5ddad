"""Learned surrogates of the sky radiance and of the camera-to-surface
in-scattering / transmittance (no counterpart in the reference).

Training data come from the plain CUDA integrator itself
(``atm_surrogate_samples``): features uniform over the input box, over a grid
of parameter sets that differ in their Rayleigh and Mie scale heights (the
networks' features 4 and 5).  Networks are trained by the package's own fused
FP32 forward/backward kernels with Adam on standardised targets; the
standardisation is then folded into the output layer and the weights are
packed for the BF16 tensor-core composite (``atm_composite_surrogate``).

Networks (feature layout in ``include/atm_capi.h``):
  * sky:    10 -> 3 x 64 SiLU -> 3  sky radiance, ln(L / E + floor)
  * aerial: 11 -> 4 x 64 SiLU -> 6  segment in-scattering (``TargetSpec``),
                                     optical depth
The surrogate composite takes the surface pixels' transmittance from the
transmittance LUT, as the plain composite does; the aerial network's
optical-depth outputs are trained and reported, not used in the frame.
"""

from __future__ import annotations

import ctypes
import dataclasses
import math
import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np
import torch

from .. import _native
from .batch import BatchedLutBuilder
from .config import EARTH_RADIUS_M, earth_baseline
from .mlp import Mlp, layer_shapes

SKY = _native.ATM_SURROGATE_SKY
AERIAL = _native.ATM_SURROGATE_AERIAL
# Rayleigh scale height min, max; Mie scale height min, max (m)
SCALE_HEIGHT_RANGE = (6000.0, 10000.0, 800.0, 1600.0)
SHAPES = {SKY: (10, 3, 3), AERIAL: (11, 4, 6)}  # n_in, hidden layers, n_out
FLOOR = 1.0e-7        # floor of the generator's targets ln(L / E + FLOOR)
MAX_LENGTH_M = 2.0e6
MAX_DEPTH = 30.0
SURFACE_RANGE_M = (-5000.0, 10000.0)  # surface altitudes of shaped aerial samples


@dataclass(frozen=True)
class TargetSpec:
    """What a network's radiance outputs mean: ln(L / E + floor + floor_t T),
    T the segment's LUT-ratio transmittance (aerial network only; the sky
    network has floor_t = 0).  A surface pixel's composite is L + C T with C
    the surface radiance behind the segment, so its error is dL / (L + C T):
    floor_t ~ C / E puts the network's relative accuracy where the frame
    needs it instead of on in-scattering too faint to see in front of the
    surface.  Outputs 3..5 of the aerial network are the optical depth."""

    floor: float = 1.0e-4
    floor_t: float = 0.0
    # loss weights (aerial): the frame's sensitivity ((L + floor) / (L + C T +
    # floor))^2 to the radiance outputs, C = surface_radiance (/ E) a lit
    # surface behind the segment; depth_weight on the optical-depth outputs.
    # 0 = unweighted.
    surface_radiance: float = 0.0
    depth_weight: float = 1.0
    # aerial sample shaping: share of training segments starting at the shell
    # top (feature 0 = 1), where every segment seen from a camera above the
    # shell starts, and share ending at a surface altitude (SURFACE_RANGE_M),
    # where every surface pixel's segment ends
    shell_top_fraction: float = 0.0
    surface_fraction: float = 0.0
    # aerial/sky sample shaping: segments start at an altitude inside this
    # band (m) - a network specialised to the cameras of that band - or
    # anywhere in the shell when None
    start_range_m: tuple | None = None
    # share of samples with the sun's zenith at the start uniform in angle in
    # [0, sun_angle_max_degrees] (the sun feature's map concentrates samples
    # on the horizon and leaves a high sun sparse)
    sun_angle_fraction: float = 0.0
    sun_angle_max_degrees: float = 100.0


# Aerial defaults from frames against FP64 (three cameras, 2 km - 2000 km):
# the frame-sensitivity weights cut the 50 km and 2000 km cameras' errors
# 2-3x (held-out averages over the uniform box hide this), and a quarter of
# the samples at the shell top serves the cameras above the shell.  The
# surface behind the segment is taken dim (C = 0.005 E, a low sun's lit
# ground): with C = 0.02 E the weights neglect the in-scattering of low-sun
# frames, whose surfaces are far dimmer (50 km camera at sun zenith 83 deg:
# 2.0% mean frame error against 1.7% with 0.005; unweighted, 2.3%).
DEFAULT_SPECS = {SKY: TargetSpec(1.0e-4), AERIAL: TargetSpec(1.0e-4, 0.0, 0.005, 0.1, 0.25, 0.6)}
# The pair of aerial networks used by train_surrogate: one for cameras inside
# the shell (its segments start anywhere below the top) and one for cameras
# above it (every segment starts at the shell top); the composite picks per
# frame.  The radiance floor must be the same for both.
AERIAL_INSIDE_SPEC = TargetSpec(1.0e-4, 0.0, 0.005, 0.1, 0.0, 0.6)
AERIAL_ABOVE_SPEC = TargetSpec(1.0e-4, 0.0, 0.002, 0.1, 1.0, 0.6)


def loss_weights(kind: int, y: torch.Tensor, spec: TargetSpec):
    """Per-output loss weights (mean 1 per output) or None."""

    if kind != AERIAL or spec.surface_radiance <= 0.0:
        return None
    L = _generator_radiance(y)
    T = torch.exp(-y[:, 3:6])
    w = ((L + spec.floor) / (L + spec.surface_radiance * T + spec.floor)) ** 2
    w = torch.cat([w, torch.full_like(w, spec.depth_weight)], 1)
    return w / w.mean(0).clamp_min(1e-12)


def _generator_radiance(y: torch.Tensor) -> torch.Tensor:
    return (torch.exp(y[:, :3]) - FLOOR).clamp_min(0.0)


def to_targets(kind: int, y: torch.Tensor, spec: TargetSpec) -> torch.Tensor:
    """Network targets from the generator's (ln(L/E + 1e-7)[, optical depth])."""

    L = _generator_radiance(y)
    if kind == SKY:
        return torch.log(L + spec.floor)
    return torch.cat([torch.log(L + spec.floor + spec.floor_t * torch.exp(-y[:, 3:6])), y[:, 3:6]], 1)


def radiance_of(kind: int, out: torch.Tensor, spec: TargetSpec, transmittance=None) -> torch.Tensor:
    """L / E of network outputs (``transmittance``: the LUT-ratio T, aerial)."""

    floor = spec.floor if kind == SKY else spec.floor + spec.floor_t * transmittance
    return (torch.exp(out[:, :3]) - floor).clamp_min(0.0)


def parameter_grid(base=None, rayleigh=(6000.0, 8000.0, 10000.0), mie=(800.0, 1200.0, 1600.0)):
    """Parameter sets of the training data: ``base`` (Earth-like by default)
    with every (Rayleigh, Mie) scale-height pair of the grid."""

    base = base or earth_baseline()
    return [dataclasses.replace(base, rayleigh_scale_height_m=float(hr), mie_scale_height_m=float(hm))
            for hr in rayleigh for hm in mie]


def scale_height_features(config, scale_height_range=SCALE_HEIGHT_RANGE):
    lo_r, hi_r, lo_m, hi_m = scale_height_range
    f = lambda h, lo, hi: 2.0 * (math.log(h) - math.log(lo)) / (math.log(hi) - math.log(lo)) - 1.0
    return f(config.rayleigh_scale_height_m, lo_r, hi_r), f(config.mie_scale_height_m, lo_m, hi_m)


class SampleSource:
    """Training samples from the plain integrator over parameter sets of one
    planet (their transmittance and multi-scattering LUTs are built once)."""

    def __init__(self, configs, planet_radius_m: float = EARTH_RADIUS_M, solar_irradiance=(4.0, 3.9, 3.7),
                 sun_angular_radius_degrees: float = 0.266, scale_height_range=SCALE_HEIGHT_RANGE, device=None):
        self.configs = list(configs)
        self.planet_radius_m = float(planet_radius_m)
        self.top_altitude_m = float(self.configs[0].top_altitude_m)
        self.scale_height_range = tuple(float(v) for v in scale_height_range)
        self.builder = BatchedLutBuilder([(c, planet_radius_m) for c in self.configs], solar_irradiance,
                                         sun_angular_radius_degrees, device=device)
        self.device = self.builder.device

    def samples(self, kind: int, n: int, seed: int, shell_top_fraction: float = 0.0, surface_fraction: float = 0.0,
                surface_range_m=SURFACE_RANGE_M, start_range_m=None, sun_angle=(0.0, 100.0)):
        """(features, targets) of n samples.  Aerial samples: a share
        ``shell_top_fraction`` starts at the shell top (feature 0 = 1) and a
        share ``surface_fraction`` ends at an altitude uniform in
        ``surface_range_m``; the rest is uniform over the input box.
        ``start_range_m`` (lo, hi) confines the start altitudes to that band
        (uniform in the altitude feature); ``sun_angle`` (share, max degrees)
        draws that share of the sun zeniths uniform in angle."""

        n_in, _, n_out = SHAPES[kind]
        x = torch.empty((n, n_in), dtype=torch.float32, device=self.device)
        y = torch.empty((n, n_out), dtype=torch.float32, device=self.device)
        rng = (ctypes.c_double * 4)(*self.scale_height_range)
        lo, hi = start_range_m if start_range_m is not None else (0.0, 0.0)
        opts = _native.AtmSampleOptions(float(shell_top_fraction), float(surface_fraction), float(surface_range_m[0]),
                                        float(surface_range_m[1]), float(lo), float(hi), float(sun_angle[0]),
                                        float(sun_angle[1]))
        _native.check(self.builder._lib.atm_surrogate_samples(
            self.builder._handle, int(kind), int(n), int(seed) & (2**64 - 1), ctypes.byref(opts), rng,
            ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), self.builder._stream()))
        return x, y

    def close(self):
        self.builder.close()


@dataclass
class TrainReport:
    kind: int
    steps: int
    batch: int
    n_samples: int
    seconds: float
    loss: list = field(default_factory=list)         # (step, mean squared error, standardised)
    held_out: dict = field(default_factory=dict)
    spec: TargetSpec | None = None


def _fold_standardisation(params: torch.Tensor, shapes, mean: torch.Tensor, std: torch.Tensor) -> torch.Tensor:
    """Parameters whose output layer returns std * y + mean."""

    p = params.clone()
    off = 0
    for i, (o, n_in) in enumerate(shapes):
        w = p[off:off + o * n_in].view(o, n_in)
        b = p[off + o * n_in:off + o * n_in + o]
        if i == len(shapes) - 1:
            w.mul_(std[:, None])
            b.mul_(std).add_(mean)
        off += o * n_in + o
    return p


def held_out_error(net: Mlp, kind: int, x: torch.Tensor, y: torch.Tensor, spec: TargetSpec,
                   precision: str = "bf16") -> dict:
    """Errors of a de-standardised network on held-out samples: radiance as
    relative error where L > 1e-4 E; for the aerial network also the
    composite-like error |dL| / (L + C T + 1e-4 E) with a lit surface of
    radiance C = 0.02 E behind the segment and the LUT-ratio T (as the
    composite uses it), and the optical-depth output's absolute error."""

    pred = net.forward(x, precision).double()
    yd = y.double()
    Lt = _generator_radiance(yd)
    Tt = torch.exp(-yd[:, 3:6]) if kind == AERIAL else None
    Lp = radiance_of(kind, pred, spec, Tt)
    bright = Lt > 1e-4
    rel = ((Lp - Lt).abs() / Lt.clamp_min(1e-30))[bright]
    q = lambda v, p: float(torch.quantile(v[:1 << 20].float(), p)) if v.numel() else 0.0
    out = {"radiance_rel_mean": float(rel.mean()) if rel.numel() else 0.0, "radiance_rel_p99": q(rel, 0.99)}
    if kind == AERIAL:
        C = 0.02
        comp = ((Lp - Lt).abs() / (Lt + C * Tt + 1e-4)).max(1).values
        out["composite_rel_mean"] = float(comp.mean())
        out["composite_rel_p99"] = q(comp, 0.99)
        dtau = (pred[:, 3:6].clamp_min(0) - yd[:, 3:6]).abs()
        live = yd[:, 3:6] < 10.0
        out["depth_abs_mean"] = float(dtau[live].mean())
    return out


def train(source: SampleSource, kind: int, n_samples: int = 2**22, batch: int = 65536, epochs: int = 200,
          lr: float = 2e-3, lr_final: float = 1e-5, seed: int = 1, held_out: int = 2**16,
          spec: TargetSpec | None = None, log_every: int = 100) -> tuple[Mlp, TrainReport]:
    """Train one surrogate network on ``n_samples`` integrator samples with
    Adam (cosine learning-rate decay from ``lr`` to ``lr_final``).  Returns
    the network (standardisation folded in, BF16 packed) and a report with
    the loss history and held-out errors."""

    spec = spec or DEFAULT_SPECS[kind]
    n_in, n_hidden, n_out = SHAPES[kind]
    x, y = source.samples(kind, n_samples, seed, spec.shell_top_fraction, spec.surface_fraction,
                          start_range_m=spec.start_range_m,
                          sun_angle=(spec.sun_angle_fraction, spec.sun_angle_max_degrees))
    t = to_targets(kind, y, spec)
    w = loss_weights(kind, y, spec)
    del y
    mean, std = t.mean(0), t.std(0).clamp_min(1e-6)
    ts = (t - mean) / std
    del t
    net = Mlp(n_in, n_hidden, n_out, seed=seed, device=source.device)
    steps_per_epoch = max(n_samples // batch, 1)
    steps = steps_per_epoch * epochs
    gen = torch.Generator(device=source.device)
    gen.manual_seed(seed)
    report = TrainReport(kind, steps, batch, n_samples, 0.0)
    torch.cuda.synchronize(source.device)
    t0 = time.perf_counter()
    step = 0
    for epoch in range(epochs):
        perm = torch.randperm(n_samples, device=source.device, generator=gen)
        for k in range(steps_per_epoch):
            idx = perm[k * batch:(k + 1) * batch]
            frac = step / max(steps - 1, 1)
            rate = lr_final + 0.5 * (lr - lr_final) * (1.0 + math.cos(math.pi * frac))
            loss = net.train_step(x[idx], ts[idx], lr=rate, weights=None if w is None else w[idx])
            if log_every and step % log_every == 0:
                report.loss.append((step, float(loss) / (batch * n_out)))
            step += 1
    torch.cuda.synchronize(source.device)
    report.seconds = time.perf_counter() - t0
    folded = _fold_standardisation(net.params(), layer_shapes(n_in, n_hidden, n_out), mean, std)
    net.set_params(folded)
    net.pack()
    # held-out: the input box (segments starting at the shell top where the
    # network serves only those), and segments ending at a surface
    xh, yh = source.samples(kind, held_out, seed + 7919, 1.0 if spec.shell_top_fraction >= 1.0 else 0.0,
                            start_range_m=spec.start_range_m)
    report.held_out = {"bf16": held_out_error(net, kind, xh, yh, spec, "bf16"),
                       "f32": held_out_error(net, kind, xh, yh, spec, "f32")}
    if kind == AERIAL and spec.surface_fraction > 0.0:  # segments ending at a surface, as the frame's
        xs, ys = source.samples(kind, held_out, seed + 7921, spec.shell_top_fraction, 1.0,
                                start_range_m=spec.start_range_m)
        report.held_out["bf16_surface"] = held_out_error(net, kind, xs, ys, spec, "bf16")
    report.spec = spec
    return net, report


class Surrogate:
    """The networks plus what atm_composite_surrogate needs to use them:
    ``aerial`` (or, for frames whose camera is above the shell,
    ``aerial_above_shell`` when given) for surface pixels, ``sky`` for sky
    pixels; any may be None (plain path)."""

    def __init__(self, aerial: Mlp | None, sky: Mlp | None, planet_radius_m: float = EARTH_RADIUS_M,
                 top_altitude_m: float = 100_000.0, scale_height_range=SCALE_HEIGHT_RANGE,
                 aerial_spec: TargetSpec | None = None, sky_spec: TargetSpec | None = None,
                 aerial_above_shell: Mlp | None = None, aerial_bands=()):
        self.aerial, self.sky, self.aerial_above_shell = aerial, sky, aerial_above_shell
        # (highest camera altitude in m, network) pairs, ascending: a camera
        # inside the shell uses the first band that reaches its altitude
        # (a network trained on segments starting in that band), else aerial
        self.aerial_bands = sorted(((float(a), net) for a, net in aerial_bands), key=lambda b: b[0])
        self.planet_radius_m = float(planet_radius_m)
        self.top_altitude_m = float(top_altitude_m)
        self.scale_height_range = tuple(float(v) for v in scale_height_range)
        self.aerial_spec = aerial_spec or DEFAULT_SPECS[AERIAL]
        self.sky_spec = sky_spec or DEFAULT_SPECS[SKY]
        for net in (aerial, sky, aerial_above_shell, *(n for _, n in self.aerial_bands)):
            if net is not None:
                net.pack()

    def aerial_for(self, camera_altitude_m: float | None):
        """The aerial network for a camera inside the shell at this altitude."""

        if camera_altitude_m is not None:
            for top, net in self.aerial_bands:
                if camera_altitude_m <= top:
                    return net
        return self.aerial

    # gates -> plain path: |sun cosine| below twilight_cosine at a surface
    # segment's start, middle or end (measured: the aerial network's frame
    # error is flat down to 0.02 and rises below it), below
    # sky_twilight_cosine at the camera for sky pixels, view ray within
    # limb_degrees of the limb
    twilight_cosine = 0.02
    sky_twilight_cosine = 0.1
    limb_degrees = 0.5
    # bound of each tensor-core completion wait: 0 = the library's; -1 = none
    # (every wait gives up at once, the MLP pixels take the plain path)
    tc_wait_polls = 0
    # gate -> plain path: a surface segment crossing the terminator (its sun
    # cosine changes sign between its start, middle and end)
    gate_terminator = False
    # calibration from the checked pixels: the side of the tiles (pixels, a
    # power of two in 16..256; 0 = off) whose checked pixels' mean log ratio
    # of plain to network in-scattering rescales the tile's other MLP pixels
    # (measured over the 64-frame 4K sweep: frame error mean 0.45% -> 0.18%,
    # worst 1.46% -> 0.43% at 64 px, nearly flat from 32 to 128)
    calibration_tile = 64

    def native(self, check_fraction: float = 0.01, seed: int = 0, stats=None,
               camera_altitude_m: float | None = None) -> _native.AtmSurrogate:
        s = _native.AtmSurrogate()
        aerial = self.aerial_for(camera_altitude_m)
        s.aerial = aerial.handle.value if aerial is not None else None
        s.sky = self.sky.handle.value if self.sky is not None else None
        s.aerial_above_shell = self.aerial_above_shell.handle.value if self.aerial_above_shell is not None else None
        s.scale_height_range[:] = list(self.scale_height_range)
        s.trained_planet_radius_m = self.planet_radius_m
        s.trained_top_altitude_m = self.top_altitude_m
        s.check_fraction = float(check_fraction)
        s.aerial_floor = float(self.aerial_spec.floor)
        s.aerial_floor_t = float(self.aerial_spec.floor_t)
        s.sky_floor = float(self.sky_spec.floor)
        s.twilight_cosine = float(self.twilight_cosine)
        s.sky_twilight_cosine = float(self.sky_twilight_cosine)
        s.limb_degrees = float(self.limb_degrees)
        s.seed = int(seed) & 0xFFFFFFFF
        s.tc_wait_polls = int(self.tc_wait_polls)
        s.gate_terminator = 1 if self.gate_terminator else 0
        s.calibration_tile = int(self.calibration_tile)
        s.stats = stats
        return s

    def save(self, directory) -> None:
        d = Path(directory)
        d.mkdir(parents=True, exist_ok=True)
        for name, net in (("aerial", self.aerial), ("sky", self.sky), ("aerial_above_shell", self.aerial_above_shell)):
            if net is not None:
                net.save(d / f"{name}.npz")
        for k, (_, net) in enumerate(self.aerial_bands):
            net.save(d / f"aerial_band{k}.npz")
        np.savez(d / "meta.npz", planet_radius_m=self.planet_radius_m, top_altitude_m=self.top_altitude_m,
                 scale_height_range=np.array(self.scale_height_range),
                 aerial_spec=np.array([self.aerial_spec.floor, self.aerial_spec.floor_t]),
                 sky_spec=np.array([self.sky_spec.floor, self.sky_spec.floor_t]),
                 band_tops_m=np.array([top for top, _ in self.aerial_bands], dtype=np.float64))

    @classmethod
    def load(cls, directory, device=None) -> "Surrogate":
        d = Path(directory)
        meta = np.load(d / "meta.npz")
        nets = {name: (Mlp.load(d / f"{name}.npz", device=device) if (d / f"{name}.npz").exists() else None)
                for name in ("aerial", "sky", "aerial_above_shell")}
        spec = lambda a: TargetSpec(float(a[0]), float(a[1]))
        tops = meta["band_tops_m"] if "band_tops_m" in meta.files else []
        bands = [(float(top), Mlp.load(d / f"aerial_band{k}.npz", device=device)) for k, top in enumerate(tops)]
        return cls(nets["aerial"], nets["sky"], float(meta["planet_radius_m"]), float(meta["top_altitude_m"]),
                   tuple(float(v) for v in meta["scale_height_range"]), spec(meta["aerial_spec"]),
                   spec(meta["sky_spec"]), nets["aerial_above_shell"], aerial_bands=bands)


# Camera-altitude bands of the aerial networks inside the shell (m).  Each
# band's network is trained on segments starting in that band; a frame picks
# the band of its camera on the host.  Specialised this way, the network of
# cameras within 100 m of the ground is ~20x more accurate in the frame than
# one network for the whole shell, and the mid-altitude bands 1.5-3x.
INSIDE_BANDS_M = ((0.0, 100.0), (100.0, 3000.0), (3000.0, 25000.0), (25000.0, 100000.0))
# Share of training samples with the sun's zenith uniform in angle (0-100
# deg): the sun feature's map puts a sun within 20 deg of the zenith into 1.5%
# of the feature range, and frames under a high sun had 2-3x the error of
# the rest without it.
SUN_ANGLE_FRACTION = 0.5


def train_surrogate(configs=None, n_samples: int = 2**22, batch: int = 16384, epochs: int = 400, seed: int = 1,
                    lr: float = 4e-3, device=None, log_every: int = 100, above_shell: bool = True,
                    bands=INSIDE_BANDS_M, sun_angle_fraction: float = SUN_ANGLE_FRACTION, sky: bool = True):
    """The networks on the default grid: one aerial network per camera
    altitude band inside the shell (``bands``; one network for the whole
    shell when empty), the aerial network for cameras above the shell
    (``above_shell``) and the sky network (``sky``).  Returns (Surrogate,
    {name: report})."""

    source = SampleSource(configs or parameter_grid(), device=device)
    reports = {}
    band_nets = []
    try:
        inside_spec = dataclasses.replace(AERIAL_INSIDE_SPEC if above_shell else DEFAULT_SPECS[AERIAL],
                                          sun_angle_fraction=sun_angle_fraction)
        if bands:
            for k, (lo, hi) in enumerate(bands):
                spec = dataclasses.replace(inside_spec, start_range_m=(float(lo), float(hi)))
                net, reports[f"aerial_{int(lo)}_{int(hi)}m"] = train(
                    source, AERIAL, n_samples, batch, epochs, lr=lr, seed=seed + 10 + k, spec=spec,
                    log_every=log_every)
                band_nets.append((float(hi), net))
            aerial = band_nets[-1][1]
        else:
            aerial, reports["aerial"] = train(source, AERIAL, n_samples, batch, epochs, lr=lr, seed=seed,
                                              spec=inside_spec, log_every=log_every)
        above = None
        if above_shell:
            above_spec = dataclasses.replace(AERIAL_ABOVE_SPEC, sun_angle_fraction=sun_angle_fraction)
            above, reports["aerial_above_shell"] = train(source, AERIAL, n_samples, batch, epochs, lr=lr,
                                                         seed=seed + 2, spec=above_spec, log_every=log_every)
        sky_net = None
        if sky:
            sky_net, reports["sky"] = train(source, SKY, n_samples, batch, epochs, lr=lr, seed=seed + 1,
                                            spec=DEFAULT_SPECS[SKY], log_every=log_every)
    finally:
        source.close()
    return Surrogate(aerial, sky_net, source.planet_radius_m, source.top_altitude_m, source.scale_height_range,
                     inside_spec, DEFAULT_SPECS[SKY], above, aerial_bands=band_nets), reports


def stats_summary(stats: torch.Tensor) -> dict:
    s = [float(v) for v in stats.cpu()]
    n = max(s[0], 1.0)
    return {"checked": int(s[0]), "check_rel_mean": s[1] / n, "check_rel_max": s[2], "gated_surface": int(s[3]),
            "mlp_surface": int(s[4]), "mlp_sky": int(s[5]), "lut_sky": int(s[6]), "tensor_core_timeouts": int(s[7])}
