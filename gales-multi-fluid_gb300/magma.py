"""Magma mixtures: the props.txt "mix_of_mix" of "magma_mix" blocks of the shipped
cases (sim/fluid_mc/P0/props.txt), their solubility lookup tables and the GPU
evaluation of the mixture properties (include/gales_asm.h, gales_magma_*).

MagmaMix holds one magma_mix block (fluid_properties_reader.hpp:293-420) with its
tables (input/lookuptable/pressure.txt, optional temperature.txt,
wf_l_h2o_onliq_<name>.txt, wf_l_co2_onliq_<name>.txt; mixtures.hpp:418-500).
MagmaMaterial uploads a list of them and evaluates fluid_properties' mixture of
sub-mixtures (fluid_properties.hpp:171-200) on the GPU, one thread per point.
"""
from __future__ import annotations

import ctypes as C
import re
from dataclasses import dataclass, field
from pathlib import Path
from typing import List, Optional, Sequence

import numpy as np

from . import abi

GAS_ON_MU = {"none": 0, "Ishii_Zuber": 1, "Pal_2003": 2}
CRYSTAL_ON_MU = {"none": 0, "Einstein_Roscoe": 1, "Caricchi": 2}
FIELDS = ("rho", "mu", "cp", "cv", "kappa", "sound_speed", "alpha", "beta")
COMP_FIELDS = ("rho", "internal_energy", "chemical_diffusivity", "gas_volume_fraction")


@dataclass
class MagmaMix:
    """One magma_mix block; defaults as fluid_properties_reader.hpp:296-301.  Model
    names other than those of GAS_ON_MU / CRYSTAL_ON_MU select no correction, as in
    magma_mixture::properties (mixtures.hpp:170-175)."""
    name: str
    oxide_wf: Sequence[float]
    h2o_wf: float = 0.0
    co2_wf: float = 0.0
    melt_kappa: float = 1.5
    h2o_l_cp: float = 2278.0
    h2o_l_kappa: float = 0.64
    co2_l_cp: float = 2278.0
    co2_l_kappa: float = 0.64
    crystal_fraction: float = 0.0
    crystal_rho: float = 0.0
    gas_on_mu: str = "none"
    crystal_on_mu: str = "none"
    p_table: Optional[np.ndarray] = None
    T_table: Optional[np.ndarray] = None
    wf_l_h2o: Optional[np.ndarray] = None
    wf_l_co2: Optional[np.ndarray] = None
    _keep: list = field(default_factory=list, repr=False)

    def with_tables(self, p_table, wf_l_h2o, wf_l_co2, T_table=None) -> "MagmaMix":
        self.p_table = np.ascontiguousarray(p_table, dtype=np.float64)
        self.T_table = None if T_table is None else np.ascontiguousarray(T_table, dtype=np.float64)
        self.wf_l_h2o = np.ascontiguousarray(wf_l_h2o, dtype=np.float64)
        self.wf_l_co2 = np.ascontiguousarray(wf_l_co2, dtype=np.float64)
        return self

    def desc(self) -> abi.MagmaDesc:
        if self.p_table is None or self.wf_l_h2o is None or self.wf_l_co2 is None:
            raise ValueError(f"magma {self.name}: lookup tables missing")
        n_T = 0 if self.T_table is None else len(self.T_table)
        n_p = len(self.p_table)
        want = n_p * max(n_T, 1)
        if self.wf_l_h2o.size != want or self.wf_l_co2.size != want:
            raise ValueError(f"magma {self.name}: tables must hold {want} values")
        dp = C.POINTER(C.c_double)
        arrs = [self.p_table, self.wf_l_h2o, self.wf_l_co2] + ([self.T_table] if n_T else [])
        self._keep = arrs
        d = abi.MagmaDesc()
        for i, v in enumerate(self.oxide_wf):
            d.oxide_wf[i] = float(v)
        for k in ("melt_kappa", "h2o_wf", "h2o_l_cp", "h2o_l_kappa", "co2_wf", "co2_l_cp", "co2_l_kappa",
                  "crystal_fraction", "crystal_rho"):
            setattr(d, k, float(getattr(self, k)))
        d.gas_on_mu = GAS_ON_MU.get(self.gas_on_mu, 0)
        d.crystal_on_mu = CRYSTAL_ON_MU.get(self.crystal_on_mu, 0)
        d.n_p, d.n_T = n_p, n_T
        d.p_table = self.p_table.ctypes.data_as(dp)
        d.T_table = self.T_table.ctypes.data_as(dp) if n_T else None
        d.wf_l_h2o = self.wf_l_h2o.ctypes.data_as(dp)
        d.wf_l_co2 = self.wf_l_co2.ctypes.data_as(dp)
        return d


@dataclass
class CustomMix:
    """A custom_mix block (custom_mixture, mixtures.hpp:69-101;
    fluid_properties_reader.hpp:222-274): a sub-mixture of constant rho, mu, cp, kappa,
    alpha and beta."""
    name: str
    rho: float
    mu: float
    cp: float
    kappa: float
    alpha: float = 0.0
    beta: float = 0.0

    def desc(self) -> abi.MagmaDesc:
        d = abi.MagmaDesc()
        d.kind = abi.SUBMIX_CUSTOM
        d.chemical.kind = abi.CH_CUSTOM
        for k in ("rho", "mu", "cp", "kappa", "alpha", "beta"):
            setattr(d.chemical, k, float(getattr(self, k)))
        d.chemical.cv = float(self.cp)
        return d


@dataclass
class ChemicalAsMix:
    """A ch_as_mix block (ch_as_mix, mixtures.hpp:25-53; fluid_properties_reader.hpp:
    175-205): one chemical (custom_chemical or ideal_gas descriptor) as a sub-mixture."""
    name: str
    chemical: abi.ChemicalDesc

    def desc(self) -> abi.MagmaDesc:
        d = abi.MagmaDesc()
        d.kind = abi.SUBMIX_CHEMICAL
        d.chemical = self.chemical
        return d


def descs(comps: Sequence[MagmaMix]):
    arr = (abi.MagmaDesc * len(comps))()
    for i, m in enumerate(comps):
        arr[i] = m.desc()
    return arr


def _addr(x):
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    return x.data_ptr()


class MagmaMaterial:
    """fluid_properties with mix_of_mix of magma mixtures, evaluated on the GPU."""

    def __init__(self, comps: Sequence[MagmaMix]):
        from . import GalesError
        self.comps = list(comps)
        self.nb_comp = len(self.comps)
        self._L = abi.lib()
        self._d = descs(self.comps)
        h = C.c_void_p()
        rc = self._L.gales_magma_create(self._d, self.nb_comp, C.byref(h))
        if rc:
            raise GalesError(rc, "gales_magma_create failed")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.gales_magma_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def properties(self, p, T, Y, shear=None, with_components: bool = False, stream: int = 0):
        """Mixture properties at the points (p[i], T[i], Y[i, :]) with all nb_comp mass
        fractions per point: a dict of FIELDS arrays (and COMP_FIELDS arrays of shape
        (nb_comp, n) with with_components).  numpy arrays or cuda tensors."""
        from . import GalesError
        is_np = isinstance(p, np.ndarray)
        if is_np:
            p = np.ascontiguousarray(p, dtype=np.float64)
            T = np.ascontiguousarray(T, dtype=np.float64)
            Y = np.ascontiguousarray(Y, dtype=np.float64)
            shear = None if shear is None else np.ascontiguousarray(shear, dtype=np.float64)
            n = len(p)
            out = np.zeros((8, n))
            comp = np.zeros((self.nb_comp, 4, n)) if with_components else None
        else:
            import torch
            n = p.numel()
            out = torch.zeros((8, n), dtype=torch.float64, device=p.device)
            comp = torch.zeros((self.nb_comp, 4, n), dtype=torch.float64, device=p.device) if with_components else None
        if Y.shape != (n, self.nb_comp):
            raise ValueError(f"Y must have shape ({n}, {self.nb_comp})")
        rc = self._L.gales_magma_properties(self._h, _addr(p), _addr(T), _addr(Y), _addr(shear), n, _addr(out),
                                            _addr(comp), stream or None)
        if rc:
            raise GalesError(rc, self._L.gales_magma_last_error(self._h).decode())
        res = {k: out[i] for i, k in enumerate(FIELDS)}
        if with_components:
            for i, k in enumerate(COMP_FIELDS):
                res["comp_" + k] = comp[:, i]
        return res


# ---------------------------------------------------------------------------
# props.txt and lookup tables

def _lines(text: str):
    """read_one_line (algorithm.hpp:219-225): trimmed, split on spaces and commas."""
    for raw in text.splitlines():
        s = raw.strip()
        yield [t for t in re.split(r"[ ,]+", s) if t] or [""]


def read_props(path) -> List[MagmaMix]:
    """The magma_mix blocks of a props.txt "fluid { mix_of_mix { ... } }"
    (fluid_properties_reader.hpp:127-156, 293-420), in file order, without tables
    (see read_lookup_tables).  Other material kinds raise ValueError."""
    it = _lines(Path(path).read_text())
    out: List[MagmaMix] = []
    for s in it:
        if s[0] in ("", "fluid", "{", "}", "mix_of_mix"):
            continue
        if s[0] != "magma_mix":
            raise ValueError(f"props.txt: unsupported entry {s[0]!r} (only mix_of_mix of magma_mix)")
        kw = {}
        for t in it:
            key = t[0]
            if key in ("", "{"):
                continue
            if key == "}":
                break
            if key == "name":
                kw["name"] = t[1]
            elif key == "oxide_wf":
                kw["oxide_wf"] = [float(v) for v in t[1:11]]
            elif key in ("gas_on_mu_model", "crystal_on_mu_model"):
                kw[key.replace("_model", "")] = t[1]
            elif key in ("melt_kappa", "h2o_wf", "h2o_l_cp", "h2o_l_kappa", "co2_wf", "co2_l_cp", "co2_l_kappa",
                         "crystal_fraction", "crystal_rho"):
                kw[key] = float(t[1])
        out.append(MagmaMix(**kw))
    return out


def _read_table(path: Path, count: Optional[int] = None):
    vals = np.array(Path(path).read_text().split(), dtype=np.float64)
    if count is not None and len(vals) < count:
        raise ValueError(f"{path}: {len(vals)} values, the table needs {count}")
    return vals if count is None else vals[:count]


def read_lookup_tables(directory, mix: MagmaMix) -> MagmaMix:
    """magma_mixture::lookup_table (mixtures.hpp:418-500): pressure.txt (count, values),
    optional temperature.txt, then wf_l_{h2o,co2}_onliq_<name>.txt ([n_T][n_p] or [n_p])."""
    d = Path(directory)
    pv = _read_table(d / "pressure.txt")
    n_p = int(pv[0])
    if len(pv) < 1 + n_p:
        raise ValueError(f"{d / 'pressure.txt'}: {len(pv) - 1} pressures, the header declares {n_p}")
    p = pv[1:1 + n_p]
    T = None
    n = n_p
    if (d / "temperature.txt").exists():
        tv = _read_table(d / "temperature.txt")
        n_T = int(tv[0])
        if len(tv) < 1 + n_T:
            raise ValueError(f"{d / 'temperature.txt'}: {len(tv) - 1} temperatures, the header declares {n_T}")
        T = tv[1:1 + n_T]
        n = len(T) * n_p
    h2o = _read_table(d / f"wf_l_h2o_onliq_{mix.name}.txt", n)
    co2 = _read_table(d / f"wf_l_co2_onliq_{mix.name}.txt", n)
    return mix.with_tables(p, h2o, co2, T)


def write_lookup_tables(directory, mix: MagmaMix):
    """Write mix's tables in the input/lookuptable format."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    fmt = lambda a: "\n".join(repr(float(v)) for v in np.ravel(a))
    (d / "pressure.txt").write_text(f"{len(mix.p_table)}\n" + fmt(mix.p_table) + "\n")
    if mix.T_table is not None:
        (d / "temperature.txt").write_text(f"{len(mix.T_table)}\n" + fmt(mix.T_table) + "\n")
    (d / f"wf_l_h2o_onliq_{mix.name}.txt").write_text(fmt(mix.wf_l_h2o) + "\n")
    (d / f"wf_l_co2_onliq_{mix.name}.txt").write_text(fmt(mix.wf_l_co2) + "\n")
