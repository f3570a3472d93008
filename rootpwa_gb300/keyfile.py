"""Wave definitions from the reference's key files and particle table.

A key file (libconfig syntax, read by waveDescription,
decayAmplitude/waveDescription.cc:495-540, :800-932) describes one wave: the
production vertex, the X quantum numbers, the decay tree with L, S and the
isobars' mass dependences, and optional amplitude options.  This module reads
the subset of libconfig that key files use (groups, lists, arrays, strings,
numbers, booleans, comments, @include) and turns the key of a three-body
decay X -> isobar + bachelor, isobar -> a + b into the arguments of
isobarHelicityAmplitudes.addWave; the isobars' masses, widths, spins and
isospins come from a particle table in the reference's format
(particleData/particleDataTable.txt: name, antiparticle, mass, width,
baryon number, 2I, S, Ch, B, G, 2J, P, C).

    table = readParticleTable("particleDataTable.txt")
    amp = isobarAmplitudesFromKeyFiles(["1-1++0+rho770_01_pi-.key", ...], table, ["pi-", "pi+", "pi-"])
"""
import os
import re

# mass dependences of the key files (decayAmplitude/massDependence.h cName)
# that the GPU amplitudes implement; an absent massDep group means the
# relativistic Breit-Wigner (massDependence.cc:115-116)
KEY_MASS_DEPENDENCES = {
    "": "relativisticBreitWigner", "flat": "flat", "relativisticBreitWigner": "relativisticBreitWigner",
    "constWidthBreitWigner": "constWidthBreitWigner", "rhoBreitWigner": "rhoBreitWigner",
    "f0980BreitWigner": "f0980BreitWigner", "f_0(980)": "f0980BreitWigner",
    "f0980FlatteBesII": "f0980FlatteBesII", "f_0(980)Flatte": "f0980FlatteBesII",
    "piPiSWaveAuMorganPenningtonM": "piPiSWaveAuMorganPenningtonM",
    "piPiSWaveAuMorganPenningtonVes": "piPiSWaveAuMorganPenningtonVes",
    "piPiSWaveAuMorganPenningtonKachaev": "piPiSWaveAuMorganPenningtonKachaev", "binned": "binned",
    "rhoPrime": "rhoPrime", "KPiSGLASS": "KPiSGLASS", "KPiSPalanoPennington": "KPiSPalanoPennington",
}
# KPiSGLASS::Create (massDependence.cc:660-686) reads these from the massDep group
GLASS_PARAMETERS = ("a", "r", "M0", "G0", "phiF", "phiR", "phiRsin", "F", "R", "MMax")


# -- libconfig subset ----------------------------------------------------------------

class _Group(list):
    """ordered (name, value) pairs of a libconfig group; the order matters
    (the X vertex's daughter order follows it, waveDescription.cc:914-923)."""

    def get(self, name, default=None):
        for k, v in self:
            if k == name:
                return v
        return default

    def index(self, name):
        for i, (k, _) in enumerate(self):
            if k == name:
                return i
        return -1


_TOKEN = re.compile(r'''\s*(?:
    (?P<str>"(?:[^"\\]|\\.)*")|
    (?P<num>[+-]?(?:0[xX][0-9a-fA-F]+|(?:\d+\.\d*|\.\d+|\d+)(?:[eE][+-]?\d+)?)L{0,2})|
    (?P<name>[A-Za-z*][-A-Za-z0-9_*]*)|
    (?P<punct>[=:;,{}()\[\]])
    )''', re.X)


def _strip_comments(text):
    out, i, n = [], 0, len(text)
    while i < n:
        c = text[i]
        if c == '"':
            j = i + 1
            while j < n and text[j] != '"':
                j += 2 if text[j] == "\\" else 1
            out.append(text[i:j + 1])
            i = j + 1
        elif text.startswith("//", i) or c == "#":
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            if j < 0:
                raise ValueError("unterminated comment")
            i = j + 2
        else:
            out.append(c)
            i += 1
    return "".join(out)


def _expand_includes(path, depth=0):
    if depth > 10:
        raise ValueError("@include nested too deeply")
    base = os.path.dirname(os.path.abspath(path))
    lines = []
    with open(path) as f:
        for line in f:
            m = re.match(r'\s*@include\s+"([^"]+)"', line)
            if m:
                inc = m.group(1)
                lines.append(_expand_includes(inc if os.path.isabs(inc) else os.path.join(base, inc), depth + 1))
            else:
                lines.append(line)
    return "".join(lines)


def _tokens(text):
    pos, out = 0, []
    text = _strip_comments(text)
    while pos < len(text):
        if text[pos:].strip() == "":
            break
        m = _TOKEN.match(text, pos)
        if not m or m.end() == pos:
            raise ValueError("libconfig: cannot parse near %r" % text[pos:pos + 30])
        for kind in ("str", "num", "name", "punct"):
            if m.group(kind) is not None:
                out.append((kind, m.group(kind)))
                break
        pos = m.end()
    return out


def _parse_value(tok, i):
    kind, val = tok[i]
    if kind == "str":
        s, j = [], i
        while j < len(tok) and tok[j][0] == "str":        # adjacent strings concatenate
            s.append(bytes(tok[j][1][1:-1], "utf-8").decode("unicode_escape"))
            j += 1
        return "".join(s), j
    if kind == "num":
        v = val.rstrip("L")
        if v.lower().startswith(("0x", "+0x", "-0x")):
            return int(v, 16), i + 1
        return (float(v) if any(c in v for c in ".eE") else int(v)), i + 1
    if kind == "name" and val.lower() in ("true", "false"):
        return val.lower() == "true", i + 1
    if val == "{":
        return _parse_group(tok, i + 1, "}")
    if val in "([":
        close = ")" if val == "(" else "]"
        items, j = [], i + 1
        while tok[j][1] != close:
            v, j = _parse_value(tok, j)
            items.append(v)
            if tok[j][1] == ",":
                j += 1
        return items, j + 1
    raise ValueError("libconfig: unexpected %r" % val)


def _parse_group(tok, i, close):
    g = _Group()
    while i < len(tok) and tok[i][1] != close:
        kind, name = tok[i]
        if kind != "name" or tok[i + 1][1] not in "=:":
            raise ValueError("libconfig: expected a setting name, got %r" % name)
        v, i = _parse_value(tok, i + 2)
        g.append((name, v))
        while i < len(tok) and tok[i][1] in ";,":
            i += 1
    if close is not None:
        if i >= len(tok):
            raise ValueError("libconfig: missing %r" % close)
        i += 1
    return g, i


def parseKeyFile(path):
    """the settings of a key file as nested ordered groups (@include resolved
    relative to the file)."""
    g, _ = _parse_group(_tokens(_expand_includes(path)), 0, None)
    return g


# -- particle table ----------------------------------------------------------------

def _charge(name):
    """charge from the name (particleDataTable.txt naming scheme): last
    character -, 0 or + (otherwise neutral); a digit before it is the magnitude."""
    if not name or name[-1] not in "-0+":
        return 0
    if name[-1] == "0":
        return 0
    mag = int(name[-2]) if len(name) > 1 and name[-2].isdigit() else 1
    return mag if name[-1] == "+" else -mag


def readParticleTable(path):
    """{name: properties} from a table in the reference's format, each row
    defining a particle and its antiparticle (charge, baryon number and
    flavours negated; 2I, G, 2J, P, C kept).  2I_3 follows from
    Gell-Mann-Nishijima: Q - (B + S + Ch + beauty) / 2."""
    table = {}
    with open(path) as f:
        for line in f:
            line = line.split("#", 1)[0].strip()
            if not line:
                continue
            c = line.split()
            if len(c) < 13:
                raise ValueError("%s: a row needs 13 columns: %r" % (path, line))
            name, anti = c[0], c[1]
            mass, width = float(c[2]), float(c[3])
            bar, I2, S, Ch, B, G, J2, P, C = (int(x) for x in c[4:13])
            for nm, sgn in ((name, 1), (anti, -1)):
                q = _charge(nm)
                Y = sgn * (bar + S + Ch + B)
                table[nm] = dict(name=nm, mass=mass, width=width, isospin=I2, isospinProj=2 * q - Y, G=G, J=J2,
                                 P=P, C=C, charge=q, baryon=sgn * bar)
    return table


# -- key file -> wave -------------------------------------------------------------

def _fs_list(v):
    return [] if v is None else list(v)


def waveFromKeyFile(path, table, fsNames):
    """(addWave keyword arguments, amplitude options) of the three-body key
    file at path; fsNames are the final-state particles in event order (a
    key's final-state particle (name, index) is the index-th particle of that
    name there)."""
    key = parseKeyFile(path)
    dv = key.get("decayVertex")
    if dv is None:
        raise ValueError("%s: no decayVertex group" % path)
    xq, xd = dv.get("XQuantumNumbers"), dv.get("XDecay")
    if xq is None or xd is None:
        raise ValueError("%s: XQuantumNumbers and XDecay are needed" % path)
    fsX, isoX = _fs_list(xd.get("fsParticles")), _fs_list(xd.get("isobars"))
    if len(fsX) != 1 or len(isoX) != 1:
        raise NotImplementedError("%s: only X -> isobar + bachelor, isobar -> a + b (three final-state particles)"
                                  % path)
    iso = isoX[0]
    fsI = _fs_list(iso.get("fsParticles"))
    if len(fsI) != 2 or iso.get("isobars"):
        raise NotImplementedError("%s: the isobar must decay into two final-state particles" % path)

    def slot(p):
        name, idx = p.get("name"), int(p.get("index", 0))
        hits = [k for k, n in enumerate(fsNames) if n == name]
        if idx >= len(hits):
            raise ValueError("%s: final-state particle %s[%d] is not in %s" % (path, name, idx, fsNames))
        return hits[idx]
    a, b, c = slot(fsI[0]), slot(fsI[1]), slot(fsX[0])
    if len({a, b, c}) != 3:
        raise ValueError("%s: final-state particles map to the same slot" % path)
    iname = iso.get("name")
    if iname not in table:
        raise ValueError("%s: isobar %r is not in the particle table" % (path, iname))
    ip = table[iname]
    md = iso.get("massDep")
    mdname = "" if md is None else md.get("name", "")
    if mdname not in KEY_MASS_DEPENDENCES:
        raise NotImplementedError("%s: mass dependence %r is not implemented on the GPU" % (path, mdname))
    kw = dict(J=int(xq.get("J")), P=int(xq.get("P")), M=int(xq.get("M")), refl=int(xq.get("refl")),
              L=int(xd.get("L", 0)), S=int(xd.get("S", 0)), isobarJ=ip["J"], isobarL=int(iso.get("L", 0)),
              isobarS=int(iso.get("S", 0)), massDependence=KEY_MASS_DEPENDENCES[mdname], isobarMass=ip["mass"],
              isobarWidth=ip["width"], isobarDaughters=(a, b), bachelor=c,
              # a bachelor listed before the isobar is the X vertex's daughter 1 (waveDescription.cc:914-923)
              bachelorFirst=xd.index("fsParticles") < xd.index("isobars"),
              isobarName=iname.replace("(", "_").replace(")", "_"), isospin=int(xq.get("isospin", 0)),
              G=int(xq.get("G", 0)), C_=int(xq.get("C", 0)), isobarIsospin=ip["isospin"])
    if mdname == "KPiSGLASS":
        missing = [k for k in GLASS_PARAMETERS if md.get(k) is None]
        if missing:
            raise ValueError("%s: KPiSGLASS needs %s" % (path, ", ".join(missing)))
        kw["massDepParams"] = tuple(float(md.get(k)) for k in GLASS_PARAMETERS)
    elif mdname == "KPiSPalanoPennington":
        kw["massDepParams"] = (float(md.get("MMax", 2.4)),)     # massDependence.cc:750-759
    if mdname == "binned":
        b = md.get("bounds")
        if not isinstance(b, list) or len(b) != 2 or not b[0] <= b[1]:
            raise ValueError("%s: a binned mass dependence needs bounds = [lower, upper]" % path)
        kw["bounds"] = (float(b[0]), float(b[1]))
    amp = key.get("amplitude") or _Group()
    opts = dict(formalism=amp.get("formalism", "helicity"), boseSymmetrize=bool(amp.get("boseSymmetrize", True)),
                isospinSymmetrize=bool(amp.get("isospinSymmetrize", True)),
                useReflectivityBasis=bool(amp.get("useReflectivityBasis", True)))
    return kw, opts


def isobarAmplitudesFromKeyFiles(paths, table, fsNames, beamName="pi-", isospinSymmetrize=None):
    """an isobarHelicityAmplitudes (or isobarCanonicalAmplitudes) holding the
    waves of the key files, with the final state and options they give (the
    options must agree between the files).  Isospin symmetrisation follows
    the keys (default on, as in the reference) unless isospinSymmetrize says
    otherwise; it needs the final-state isospins, taken from the table."""
    from . import isobar as I
    waves = [waveFromKeyFile(p, table, fsNames) for p in paths]
    opts = waves[0][1]
    if any(o != opts for _, o in waves):
        raise ValueError("the key files' amplitude options differ")
    if opts["formalism"] not in ("helicity", "canonical"):
        raise NotImplementedError("formalism %r" % opts["formalism"])
    A = I.isobarCanonicalAmplitudes() if opts["formalism"] == "canonical" else I.isobarHelicityAmplitudes()
    for n in fsNames + [beamName]:
        if n not in table:
            raise ValueError("particle %r is not in the particle table" % n)
    A.setFinalState(fsNames, [table[n]["mass"] for n in fsNames], table[beamName]["mass"],
                    isospins=[(table[n]["isospin"], table[n]["isospinProj"], table[n]["P"]) for n in fsNames])
    A.enableReflectivityBasis(opts["useReflectivityBasis"])
    A.enableBoseSymmetrization(opts["boseSymmetrize"])
    iso = opts["isospinSymmetrize"] if isospinSymmetrize is None else isospinSymmetrize
    A.enableIsospinSymmetrization(iso)
    for kw, _ in waves:
        A.addWave(**kw)
    return A
