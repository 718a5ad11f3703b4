"""Reader for pseudopotentials in the psp8 format (ONCVPSP output, pspcod 8).

Produces the per-type radial tables that the reference keeps in PSD_OBJ
(src/include/isddft.h) after read_pseudopotential_PSP (src/readfiles.c:1957-2330), with the
same post-processing, so that the set-up entry points of the library see the numbers the
reference would:

* nonlocal radial parts are stored divided by r, ``UdV = u_l(r) / r``, and the r = 0 entry is
  replaced by the r = h entry (readfiles.c:2126-2131);
* the local potential is stored as ``rVloc = r * Vloc(r)``, with ``Vloc_0 = Vloc(0)``;
* the model core density (only when fchrg > 0) and the isolated-atom valence density are
  divided by 4*pi (readfiles.c:2219-2233);
* the projector cut-off ``rc[l]`` grows to the largest radius where ``|UdV| > 1e-8``
  (readfiles.c:2262-2276);
* ``is_r_uniform`` records whether the radial mesh is uniform to 1e-12.

The file layout (ABINIT's psp8) is: a title line whose first token is the element symbol and
which may carry ``r_core=`` radii; ``zatom zion pspd``; ``pspcod pspxc lmax lloc mmax r2well``;
``rchrg fchrg qchrg``; ``nproj`` per l; ``extension_switch``; then, for each l in 0..lmax, a
block header ``l  ekb_1 .. ekb_nproj`` followed by mmax rows ``i r u_1 .. u_nproj`` (the block
of l == lloc, if lloc <= lmax, holds ``i r Vloc`` instead); a block ``4`` with ``i r Vloc``
when lloc > lmax; mmax rows of the model core density when fchrg > 0; and mmax rows
``i r rho_val d1 d2`` of the valence density.
"""
import math

import numpy as np

TOL = 1e-12


class Psp8Error(ValueError):
    pass


def _numbers(tokens, i, n):
    return [float(t.replace("D", "E").replace("d", "e")) for t in tokens[i:i + n]], i + n


def read_psp8(path, element=None):
    """Parse a psp8 file. Returns a dict with the fields of the reference's PSD_OBJ:
    size, lmax, lloc, ppl, Znucl (valence charge), Zatom, pspxc, Vloc_0, fchrg, rc,
    RadialGrid, UdV (sum(ppl) x size), rVloc, rhoIsoAtom, rho_c_table, Gamma,
    is_r_uniform. `element`, if given, must match the title's first token (case-blind)."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    if len(lines) < 7:
        raise Psp8Error(f"{path}: too short for a psp8 file")
    title = lines[0].split()
    if element is not None and title[0].lower() != element.lower():
        raise Psp8Error(f"{path}: element {title[0]} does not match {element}")
    zatom, zion = (float(v) for v in lines[1].split()[:2])
    hdr = lines[2].split()
    pspcod, pspxc, lmax, lloc, mmax = (int(v) for v in hdr[:5])
    if pspcod != 8:
        raise Psp8Error(f"{path}: pspcod {pspcod} is not 8")
    rchrg, fchrg, qchrg = (float(v) for v in lines[3].split()[:3])
    nproj_line = lines[4].split()
    ppl = np.array([int(v) for v in nproj_line[:lmax + 1]], dtype=np.int32)
    ext = int(lines[5].split()[0])
    if ext in (2, 3):
        raise Psp8Error(f"{path}: spin-orbit psp8 files are not supported")
    # projector cut-off radii from the title (r_core= r_0 .. r_lmax)
    rc = np.zeros(lmax + 1)
    if "r_core=" in title:
        k = title.index("r_core=")
        for l in range(lmax + 1):
            rc[l] = float(title[k + 1 + l])

    tokens = " ".join(lines[6:]).split()
    n = mmax
    nproj = int(ppl.sum())
    lpos = np.concatenate([[0], np.cumsum(ppl)]).astype(int)
    grid = np.zeros(n)
    udv = np.zeros((nproj, n))
    rvloc = np.zeros(n)
    gamma = np.zeros(nproj)
    vloc0 = 0.0
    i = 0

    def read_local(i):
        nonlocal vloc0
        for jj in range(n):
            (_, r, v), i = _numbers(tokens, i, 3)
            grid[jj] = r
            rvloc[jj] = r * v
            if jj == 0:
                vloc0 = v
        return i

    for l in range(lmax + 1):
        l_read = int(tokens[i]); i += 1
        if l_read != l:
            raise Psp8Error(f"{path}: expected the block of l={l}, found {l_read}")
        if l != lloc:
            g, i = _numbers(tokens, i, int(ppl[l]))
            gamma[lpos[l]:lpos[l + 1]] = g
            for jj in range(n):
                vals, i = _numbers(tokens, i, 2 + int(ppl[l]))
                grid[jj] = vals[1]
                for kk in range(int(ppl[l])):
                    udv[lpos[l] + kk, jj] = vals[2 + kk] / grid[jj] if grid[jj] != 0 else 0.0
            for kk in range(int(ppl[l])):
                udv[lpos[l] + kk, 0] = udv[lpos[l] + kk, 1]
        else:
            i = read_local(i)
    if lloc > lmax:
        l_read = int(tokens[i]); i += 1
        if l_read != 4:
            raise Psp8Error(f"{path}: expected the local block (4), found {l_read}")
        i = read_local(i)

    rho_c = np.zeros(n)
    if fchrg > TOL:
        for jj in range(n):
            vals, i = _numbers(tokens, i, 7)
            rho_c[jj] = vals[2] / (4.0 * math.pi)
    rho_iso = np.zeros(n)
    for jj in range(n):
        vals, i = _numbers(tokens, i, 5)
        rho_iso[jj] = vals[2] / (4.0 * math.pi)

    if n < 2:
        raise Psp8Error(f"{path}: radial grid has fewer than 2 points")
    dr = np.diff(grid)
    if np.any(np.abs(dr) < TOL):
        raise Psp8Error(f"{path}: repeated radial grid point")
    is_uniform = int(np.all(np.abs(dr - dr[0]) <= TOL))

    # grow rc[l] to cover every |UdV| > 1e-8 beyond it
    for l in range(lmax + 1):
        if l == lloc:
            continue
        r_read = rc[l]
        for kk in range(int(ppl[l])):
            row = udv[lpos[l] + kk]
            mask = (grid > r_read) & (np.abs(row) > 1e-8)
            if mask.any():
                rc[l] = max(rc[l], float(grid[mask].max()))

    return dict(size=n, lmax=lmax, lloc=lloc, ppl=ppl, Znucl=int(zion), Zatom=int(zatom),
                pspxc=pspxc, Vloc_0=vloc0, fchrg=fchrg, rchrg=rchrg, qchrg=qchrg, rc=rc,
                RadialGrid=grid, UdV=udv, rVloc=rvloc, rhoIsoAtom=rho_iso,
                rho_c_table=rho_c, Gamma=gamma, is_r_uniform=is_uniform)


def save_tables(psd, path):
    """Write the tables of read_psp8 to an .npz file."""
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in psd.items()})


def load_tables(path):
    """Inverse of save_tables."""
    d = np.load(path)
    out = {k: d[k] for k in d.files}
    for k in ("size", "lmax", "lloc", "Znucl", "Zatom", "pspxc", "is_r_uniform"):
        out[k] = int(out[k])
    for k in ("Vloc_0", "fchrg", "rchrg", "qchrg"):
        out[k] = float(out[k])
    return out
