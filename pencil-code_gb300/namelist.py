"""Reading the reference's start.in / run.in namelists into a parameter block.

Fortran namelist groups (`&name key=value, ... /`) as read by
src/param_io.f90:82-250, :461-570, restricted to the keys of this hot path:

  &init_pars            xyz0, Lxyz, lperi, bcx, bcy, bcz ('p', 's', 'a', 'a2', 'lower:upper')
  &eos_init_pars        gamma, cs0, rho0, cp
  &run_pars             dt, nt, cdt, cdtv, itorder (3 only), it1, lbidiagonal_derij (T only),
                        bcx, bcy, bcz (override start.in's)
  &viscosity_run_pars   nu, ivisc ('nu-const' only)
  &magnetic_run_pars    eta, b_ext (B_ext), iresistivity ('eta-const' only)
  &entropy_run_pars     chi, iheatcond ('chi-const' only), lviscosity_heat
  &hydro_run_pars       lforcing_cont_uu, ampl_fcont_uu, lupw_uu
  &density_run_pars     lupw_lnrho
  &forcing_run_pars     lforcing_cont, iforcing_cont ('ABC'), ampl_ff, k1_ff, kf_fcont, relhel,
                        ABC_A, ABC_B, ABC_C; iforce ('helical' or 'zero'), force,
                        lmagnetic_forcing (with lhydro_forcing=T, crosshel=0)
  &magnetic_init_pars   initaa, amplaa (initial condition, returned separately)

Keys outside this set are kept in ``extra`` so a caller can see what was not applied.
"""
from __future__ import annotations

import re

from .lib import BC_CODES, Params, default_params

# one lexical item of a namelist body: a group start, a quoted string, the
# group terminator '/', '=', ',' or a bare word (name, index, number, logical)
_TOKEN = re.compile(r"""&\w+|'[^']*'|"[^"]*"|/|=|,|[^,\s=/'"]+""")


def _value(tok: str):
    t = tok.strip()
    if t[:1] in "'\"":
        return t[1:-1]
    low = t.lower()
    if low in (".true.", "t", "true"):
        return True
    if low in (".false.", "f", "false"):
        return False
    if "*" in t:   # repeat count r*v
        r, v = t.split("*", 1)
        return [_value(v)] * int(r)
    try:
        return int(t)
    except ValueError:
        pass
    try:
        return float(t.replace("d", "e").replace("D", "e"))
    except ValueError:
        return t


def _strip_comments(text: str) -> str:
    """Drop '!' comments that stand outside quoted strings."""
    lines = []
    for ln in text.splitlines():
        out, q = [], None
        for ch in ln:
            if q:
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
            elif ch == "!":
                break
            out.append(ch)
        lines.append("".join(out))
    return "\n".join(lines)


def parse_namelists(text: str) -> dict:
    """{group: {key: value-or-list}}; a key may carry an index, e.g. 'ampl_ff(1)'.

    Groups run from '&name' to an unquoted '/'; 'key = v1, v2, ...' lists, 'r*v'
    repeats, logicals (T/F/.true./.false.), Fortran 'd' exponents and quoted
    strings follow the namelist rules gfortran reads them with.
    """
    groups, vals, key, cur, name = {}, None, None, [], None
    toks = _TOKEN.findall(_strip_comments(text))
    i = 0
    while i < len(toks):
        t = toks[i]
        if t.startswith("&"):
            name, vals, key, cur = t[1:].lower(), {}, None, []
        elif vals is None:
            pass                                   # text outside any group
        elif t == "/":
            if key is not None:
                vals[key] = cur[0] if len(cur) == 1 else cur
            groups[name] = vals
            vals, key = None, None
        elif i + 1 < len(toks) and toks[i + 1] == "=":
            if key is not None:
                vals[key] = cur[0] if len(cur) == 1 else cur
            key, cur = t.lower(), []
            i += 1
        elif t != ",":
            v = _value(t)
            cur.extend(v if isinstance(v, list) else [v])
        i += 1
    if vals is not None:
        raise ValueError(f"namelist group &{name} has no terminating '/'")
    return groups


def _first(v):
    return v[0] if isinstance(v, list) else v


def _listed(v) -> list:
    return v if isinstance(v, list) else [v]


def _boundary_conditions(p, init: dict, run: dict) -> None:
    """lperi and bcx/bcy/bcz (cdata.f90 defaults: periodic, 'p'); run.in's bc lists
    override start.in's.  Codes of this path: 'p', 's', 'a', 'a2', as 'lower:upper'
    or one code for both sides; fields beyond the list keep 'p'."""
    nf = 8 if p.lentropy else 7
    lperi = [bool(v) for v in _listed(init.get("lperi", [True, True, True]))]
    for d, key in enumerate(("bcx", "bcy", "bcz")):
        per = lperi[d] if d < len(lperi) and lperi[d] is not None else True
        vals = run.get(key, init.get(key))
        entries = [str(v).strip().lower() for v in _listed(vals)][:nf] if vals is not None else []
        entries += ["p"] * (nf - len(entries))
        for e in entries:
            for side in e.split(":"):
                if side.strip() not in BC_CODES:
                    raise ValueError(f"{key}={e!r}: only the boundary conditions p, s, a, a2 are implemented")
        if per and any(e != "p" for e in entries):
            raise ValueError(f"{key}={entries}: non-periodic conditions on a periodic direction (lperi=T)")
        if not per and any("p" in e.split(":") for e in entries):
            raise ValueError(f"{key}={entries}: lperi=F needs a non-periodic condition for every field")
        p.set_bc(d, entries)


def params_from_namelists(start_text: str, run_text: str, n=(32, 32, 32), lentropy: int = 0,
                          precision: int = 8) -> tuple[Params, dict, dict]:
    """Parameter block of a run; returns (params, initial-condition keys, keys not applied)."""
    g = parse_namelists(start_text)
    g.update({k: v for k, v in parse_namelists(run_text).items()})
    sg = parse_namelists(start_text)
    p = default_params(nx=n[0], ny=n[1], nz=n[2], lentropy=lentropy, precision=precision)
    extra = {}

    def take(group, key, setter):
        grp = g.get(group, {})
        for k in list(grp):
            base = re.sub(r"\(.*\)$", "", k)
            if base == key:
                setter(grp[k])

    eos = sg.get("eos_init_pars", {})
    if "gamma" in eos: p.gamma = float(eos["gamma"])
    if "cs0" in eos: p.cs0 = float(eos["cs0"])
    if "rho0" in eos: p.rho0 = float(eos["rho0"])
    if "cp" in eos: p.cp = float(eos["cp"])
    init = sg.get("init_pars", {})
    if "xyz0" in init: p.xyz0[:] = [float(v) for v in init["xyz0"]]
    if "lxyz" in init: p.Lxyz[:] = [float(v) for v in init["lxyz"]]
    _boundary_conditions(p, init, g.get("run_pars", {}))
    rp = g.get("run_pars", {})
    if "dt" in rp: p.dt = float(rp["dt"])
    if "cdt" in rp: p.cdt = float(rp["cdt"])
    if "cdtv" in rp: p.cdtv = float(rp["cdtv"])
    if "itorder" in rp and int(rp["itorder"]) != 3:
        raise ValueError("only itorder=3 (2N-RK3) is implemented")
    if "lbidiagonal_derij" in rp and not rp["lbidiagonal_derij"]:
        raise ValueError("only the bidiagonal mixed derivative (lbidiagonal_derij=T) is implemented")
    take("viscosity_run_pars", "nu", lambda v: setattr(p, "nu", float(_first(v))))
    take("magnetic_run_pars", "eta", lambda v: setattr(p, "eta", float(_first(v))))
    take("magnetic_run_pars", "b_ext", lambda v: p.b_ext.__setitem__(slice(0, 3), [float(x) for x in v]))
    take("entropy_run_pars", "chi", lambda v: setattr(p, "chi", float(_first(v))))
    take("entropy_run_pars", "lviscosity_heat", lambda v: setattr(p, "lviscosity_heat", int(bool(v))))
    take("hydro_run_pars", "ampl_fcont_uu", lambda v: setattr(p, "ampl_fcont_uu", float(_first(v))))
    take("hydro_run_pars", "lupw_uu", lambda v: setattr(p, "lupw_uu", int(bool(v))))
    take("density_run_pars", "lupw_lnrho", lambda v: setattr(p, "lupw_lnrho", int(bool(v))))
    fr = g.get("forcing_run_pars", {})
    hr = g.get("hydro_run_pars", {})
    cont = bool(fr.get("lforcing_cont", False)) and bool(hr.get("lforcing_cont_uu", False))
    kinds = [str(v).strip().lower() for k, v in fr.items() if k.startswith("iforcing_cont")]
    if cont and kinds and kinds[0] != "abc":
        raise ValueError(f"continuous forcing {kinds[0]!r}: only 'ABC' is implemented")
    p.lforcing_cont = int(cont)
    iforce = str(fr.get("iforce", "zero")).strip().lower()
    if iforce not in ("zero", "helical", "2"):
        raise ValueError(f"iforce={iforce!r}: only 'helical' (and 'zero') are implemented")
    p.lforcing_hel = int(iforce in ("helical", "2"))
    take("forcing_run_pars", "force", lambda v: setattr(p, "force_hel", float(_first(v))))
    take("forcing_run_pars", "ampl_ff", lambda v: setattr(p, "ampl_ff", float(_first(v))))
    take("forcing_run_pars", "k1_ff", lambda v: setattr(p, "kf", float(_first(v))))
    take("forcing_run_pars", "kf_fcont", lambda v: setattr(p, "kf", float(_first(v))))
    take("forcing_run_pars", "relhel", lambda v: setattr(p, "relhel", float(_first(v))))
    take("forcing_run_pars", "abc_a", lambda v: setattr(p, "abc_a", float(_first(v))))
    take("forcing_run_pars", "abc_b", lambda v: setattr(p, "abc_b", float(_first(v))))
    take("forcing_run_pars", "abc_c", lambda v: setattr(p, "abc_c", float(_first(v))))
    take("forcing_run_pars", "lmagnetic_forcing", lambda v: setattr(p, "lmagnetic_forcing", int(bool(v))))
    if p.lmagnetic_forcing and not p.lforcing_hel:
        raise ValueError("lmagnetic_forcing is implemented for iforce='helical' only")
    # forcing of the vector potential as forcing_hel does it with the defaults
    # lhydro_forcing=T, crosshel=0, lforcing2_same=F, lforcing2_curl=F
    for key, default in (("lhydro_forcing", True), ("crosshel", 0.0), ("lforcing2_same", False),
                         ("lforcing2_curl", False)):
        if key in fr and _first(fr[key]) != default:
            raise ValueError(f"{key}={_first(fr[key])!r}: only the default {default!r} is implemented")
    known = {"run_pars": {"dt", "nt", "cdt", "cdtv", "itorder", "it1", "lbidiagonal_derij", "cvsid", "isave",
                          "dsnap", "dvid", "dspec", "ou_spec", "ab_spec", "lpencil_check", "bcx", "bcy", "bcz"},
             "viscosity_run_pars": {"nu", "ivisc"}, "magnetic_run_pars": {"eta", "b_ext", "iresistivity"},
             "entropy_run_pars": {"chi", "iheatcond", "lviscosity_heat"},
             "hydro_run_pars": {"lforcing_cont_uu", "ampl_fcont_uu", "lupw_uu"},
             "density_run_pars": {"lupw_lnrho"},
             "forcing_run_pars": {"lforcing_cont", "iforcing_cont", "ampl_ff", "k1_ff", "kf_fcont", "relhel",
                                  "abc_a", "abc_b", "abc_c", "iforce", "force", "lmagnetic_forcing",
                                  "lhydro_forcing", "crosshel", "lforcing2_same", "lforcing2_curl"}}
    for grp, keys in known.items():
        for k, v in g.get(grp, {}).items():
            if re.sub(r"\(.*\)$", "", k) not in keys:
                extra[f"{grp}.{k}"] = v
    ic = dict(sg.get("magnetic_init_pars", {}))
    ic.update({f"hydro.{k}": v for k, v in sg.get("hydro_init_pars", {}).items()})
    ic["nt"] = rp.get("nt")
    ic["it1"] = rp.get("it1", 10)
    ic["dsnap"] = float(_first(rp.get("dsnap", 0.0)))
    return p, ic, extra


def read_kdat(path: str):
    """The wavevector list of the random helical forcing, the reference's k.dat
    (forcing.f90:888-900): 'nk kav', then kkx, kky, kkz.  Returns ((3, nk) array, kav)
    for Box.set_kvectors / pcgb_set_kvectors."""
    import numpy as np
    with open(path) as fh:
        vals = fh.read().split()
    nk, kav = int(vals[0]), float(vals[1])
    return np.array([float(v) for v in vals[2:2 + 3 * nk]]).reshape(3, nk), kav


def kvector_shell(k2min: int, k2max: int):
    """The integer wavevectors with k2min <= |k|^2 <= k2max, in the order the
    reference's k.dat files list them (kx, then ky, then kz ascending), and their
    mean |k| (kav).  The forcing shells of the reference's samples are of this
    form: |k|^2 in [8, 12] is samples/helical-MHDturb/k.dat (98 vectors) and
    [3577, 3624] the 17550 vectors of its 4096^3 timing run."""
    import numpy as np
    kmax = int(np.floor(np.sqrt(k2max)))
    g = np.arange(-kmax, kmax + 1)
    kx, ky, kz = np.meshgrid(g, g, g, indexing="ij")
    k2 = kx * kx + ky * ky + kz * kz
    sel = (k2 >= k2min) & (k2 <= k2max)
    kvec = np.stack([kx[sel], ky[sel], kz[sel]]).astype(np.float64)
    if kvec.shape[1] == 0:
        raise ValueError(f"no integer wavevector with {k2min} <= |k|^2 <= {k2max}")
    return kvec, float(np.sqrt(k2[sel]).mean())
