"""Key files and the particle table in the reference's formats
(decayAmplitude/waveDescription.cc:495-540, :800-932;
particleData/particleDataTable.txt): the libconfig subset, the table's
antiparticles and isospin projections, three-body keys to waves and options,
and refusals of what the GPU amplitudes do not cover."""
import textwrap

import pytest

from rootpwa_gb300 import keyfile

TABLE = textwrap.dedent("""\
    # particle       antiparticle     mass         width       baryon #    2I    S    Ch   B     G    2J     P     C
    pi+              pi-              0.13957      0           0            2    0    0    0    -1     0    -1     0
    pi0              pi0              0.13498      0           0            2    0    0    0    -1     0    -1    +1
    rho(770)         rho(770)         0.7690       0.1509      0            2    0    0    0    +1     2    -1    -1
    rho(770)-        rho(770)+        0.7665       0.1502      0            2    0    0    0    +1     2    -1     0
    f2(1270)         f2(1270)         1.2751       0.1851      0            0    0    0    0    +1     4    +1    +1
    f0(980)          f0(980)          0.99         0.07        0            0    0    0    0    +1     0    +1    +1
    K+               K-               0.49368      0           0            1    1    0    0     0     0    -1     0
    """)

# a 1++ 0+ rho(770) pi S-wave, bachelor listed first (the reference's layout)
KEY_RHO = textwrap.dedent("""\
    // 1-(1++)0+ rho(770) pi S
    productionVertex : { type = "diffractiveDissVertex"; beam : { name = "pi-"; }; target : { name = "p+"; }; };
    decayVertex :
    {
      XQuantumNumbers : { isospin = 2; G = -1; J = 2; P = +1; C = +1; M = 0; refl = +1; };
      XDecay :
      {
        fsParticles = ( { name = "pi-"; index = 0; } );
        L = 0;
        S = 2;
        isobars = ( {
          name = "rho(770)";
          fsParticles = ( { name = "pi+"; }, { name = "pi-"; index = 1; } );  /* pi+ first: the analyser */
          L = 2; S = 0;
        } );
      };
    };
    """)

KEY_F2 = textwrap.dedent("""\
    decayVertex : {
      XQuantumNumbers : { isospin = 2; G = -1; J = 4; P = -1; C = +1; M = 2; refl = +1; };
      XDecay : {
        isobars = ( { name = "f2(1270)"; fsParticles = ( { name = "pi-"; index = 1; }, { name = "pi+"; } );
                      L = 4; S = 0; massDep : { name = "constWidthBreitWigner"; }; } );
        fsParticles = ( { name = "pi-"; } );
        L = 0; S = 4;
      };
    };
    @include "options.key"
    """)

OPTIONS = 'amplitude : { formalism = "canonical"; boseSymmetrize = false; isospinSymmetrize = false; }; # end\n'


@pytest.fixture
def files(tmp_path):
    (tmp_path / "table.txt").write_text(TABLE)
    (tmp_path / "rho.key").write_text(KEY_RHO)
    (tmp_path / "f2.key").write_text(KEY_F2)
    (tmp_path / "options.key").write_text(OPTIONS)
    return tmp_path


def test_libconfig_subset(tmp_path):
    p = tmp_path / "k.key"
    p.write_text('a = 1; b : { c = "x" "y"; d = [1.5, -2e3]; e = ( { f = true; }, { f = false; } ); };\n'
                 '/* block\ncomment */ g = 0x1F; // tail\n')
    k = keyfile.parseKeyFile(p)
    assert k.get("a") == 1 and k.get("g") == 31
    b = k.get("b")
    assert b.get("c") == "xy" and b.get("d") == [1.5, -2000.0]
    assert [e.get("f") for e in b.get("e")] == [True, False]
    assert [n for n, _ in b] == ["c", "d", "e"]          # order kept


def test_particle_table(files):
    t = keyfile.readParticleTable(files / "table.txt")
    assert t["pi-"]["charge"] == -1 and t["pi-"]["isospinProj"] == -2 and t["pi+"]["isospinProj"] == 2
    assert t["pi0"]["isospinProj"] == 0 and t["pi-"]["mass"] == 0.13957
    assert t["rho(770)"]["J"] == 2 and t["rho(770)"]["isospin"] == 2 and t["rho(770)+"]["charge"] == 1
    assert t["K-"]["isospinProj"] == -1 and t["K+"]["isospinProj"] == 1      # 2I_3 = 2Q - S


def test_three_body_keys_to_waves(files):
    t = keyfile.readParticleTable(files / "table.txt")
    fs = ["pi-", "pi+", "pi-"]
    kw, opts = keyfile.waveFromKeyFile(files / "rho.key", t, fs)
    assert (kw["J"], kw["P"], kw["M"], kw["refl"], kw["L"], kw["S"]) == (2, 1, 0, 1, 0, 2)
    assert (kw["isobarJ"], kw["isobarL"], kw["isobarS"], kw["isobarIsospin"]) == (2, 2, 0, 2)
    assert kw["isobarDaughters"] == (1, 2) and kw["bachelor"] == 0 and kw["bachelorFirst"]
    assert kw["massDependence"] == "relativisticBreitWigner"            # no massDep group
    assert (kw["isobarMass"], kw["isobarWidth"]) == (0.7690, 0.1509)
    assert opts == dict(formalism="helicity", boseSymmetrize=True, isospinSymmetrize=True,
                        useReflectivityBasis=True)
    kw, opts = keyfile.waveFromKeyFile(files / "f2.key", t, fs)
    assert kw["isobarDaughters"] == (2, 1) and kw["bachelor"] == 0 and not kw["bachelorFirst"]
    assert kw["massDependence"] == "constWidthBreitWigner" and kw["isobarIsospin"] == 0
    assert opts["formalism"] == "canonical" and not opts["boseSymmetrize"] and not opts["isospinSymmetrize"]


def test_amplitude_object_from_keys(files):
    t = keyfile.readParticleTable(files / "table.txt")
    A = keyfile.isobarAmplitudesFromKeyFiles([files / "rho.key"], t, ["pi-", "pi+", "pi-"])
    assert A.nmbWaves() == 1 and A.isospinSymmetrization() and A.boseSymmetrization()
    assert A.nmbSymTerms(0) == 2                   # one isospin term x two Bose terms
    assert A.waveName(0) == "[1-,1++,0+]=[pi-[0,1]rho_770_=[pi+[1,0]pi-]]"
    with pytest.raises(ValueError, match="differ"):
        keyfile.isobarAmplitudesFromKeyFiles([files / "rho.key", files / "f2.key"], t, ["pi-", "pi+", "pi-"])


def test_refusals(files, tmp_path):
    t = keyfile.readParticleTable(files / "table.txt")
    five = KEY_RHO.replace('fsParticles = ( { name = "pi+"; }, { name = "pi-"; index = 1; } );',
                           'fsParticles = ( { name = "pi+"; } ); isobars = ( { name = "rho(770)"; '
                           'fsParticles = ( { name = "pi+"; }, { name = "pi-"; } ); } );')
    (tmp_path / "four.key").write_text(five)
    with pytest.raises(NotImplementedError):
        keyfile.waveFromKeyFile(tmp_path / "four.key", t, ["pi-", "pi+", "pi-"])
    (tmp_path / "md.key").write_text(KEY_RHO.replace("L = 2; S = 0;", 'L = 2; S = 0; massDep : { name = '
                                                     '"someOtherMassDependence"; };'))
    with pytest.raises(NotImplementedError, match="someOtherMassDependence"):
        keyfile.waveFromKeyFile(tmp_path / "md.key", t, ["pi-", "pi+", "pi-"])
    (tmp_path / "iso.key").write_text(KEY_RHO.replace('name = "rho(770)"', 'name = "rho(1450)"'))
    with pytest.raises(ValueError, match="particle table"):
        keyfile.waveFromKeyFile(tmp_path / "iso.key", t, ["pi-", "pi+", "pi-"])
    with pytest.raises(ValueError, match="not in"):
        keyfile.waveFromKeyFile(files / "rho.key", t, ["pi-", "pi+", "pi0"])


def test_binned_mass_dependence_key(files, tmp_path):
    """a freed isobar: massDep { name = "binned"; bounds = [lower, upper]; }
    (massDependence.cc:187-210)."""
    t = keyfile.readParticleTable(files / "table.txt")
    key = KEY_RHO.replace('name = "rho(770)"', 'name = "f0(980)"').replace(
        "L = 2; S = 0;", 'L = 0; S = 0; massDep : { name = "binned"; bounds = [0.6, 0.9]; };').replace(
        "XQuantumNumbers : { isospin = 2; G = -1; J = 2; P = +1; C = +1; M = 0; refl = +1; };",
        "XQuantumNumbers : { isospin = 2; G = -1; J = 0; P = -1; C = +1; M = 0; refl = +1; };").replace(
        "S = 2;", "S = 0;")
    (tmp_path / "bin.key").write_text(key)
    kw, _ = keyfile.waveFromKeyFile(tmp_path / "bin.key", t, ["pi-", "pi+", "pi-"])
    assert kw["massDependence"] == "binned" and kw["bounds"] == (0.6, 0.9)
    (tmp_path / "bad.key").write_text(key.replace("[0.6, 0.9]", "[0.9, 0.6]"))
    with pytest.raises(ValueError, match="bounds"):
        keyfile.waveFromKeyFile(tmp_path / "bad.key", t, ["pi-", "pi+", "pi-"])


def test_kpi_s_wave_keys(files, tmp_path):
    """KPiSGLASS takes its ten parameters from the massDep group
    (massDependence.cc:660-686); KPiSPalanoPennington its MMax (default 2.4)."""
    t = keyfile.readParticleTable(files / "table.txt")
    glass = ('massDep : { name = "KPiSGLASS"; a = 1.95; r = 1.76; M0 = 1.435; G0 = 0.279; phiF = 0.0; '
             'phiR = 0.0; phiRsin = 0.0; F = 1.0; R = 1.0; MMax = 1.9; tag = "lass"; };')
    (tmp_path / "g.key").write_text(KEY_RHO.replace("L = 2; S = 0;", "L = 2; S = 0; " + glass))
    kw, _ = keyfile.waveFromKeyFile(tmp_path / "g.key", t, ["pi-", "pi+", "pi-"])
    assert kw["massDependence"] == "KPiSGLASS" and kw["massDepParams"] == (1.95, 1.76, 1.435, 0.279, 0.0, 0.0,
                                                                         0.0, 1.0, 1.0, 1.9)
    (tmp_path / "p.key").write_text(KEY_RHO.replace("L = 2; S = 0;", 'L = 2; S = 0; massDep : { name = '
                                                    '"KPiSPalanoPennington"; };'))
    kw, _ = keyfile.waveFromKeyFile(tmp_path / "p.key", t, ["pi-", "pi+", "pi-"])
    assert kw["massDepParams"] == (2.4,)
    (tmp_path / "bad.key").write_text(KEY_RHO.replace("L = 2; S = 0;", 'L = 2; S = 0; massDep : { name = '
                                                      '"KPiSGLASS"; a = 1.0; };'))
    with pytest.raises(ValueError, match="KPiSGLASS needs"):
        keyfile.waveFromKeyFile(tmp_path / "bad.key", t, ["pi-", "pi+", "pi-"])
