// defaults_yml.cpp - built-in defaults of the hot-path YAML sections.
// Values are the reference's defaults (src/freeform/defaults.yml:1-267 for the
// amino-acid data, :276-422 for the force terms); sections outside the hot
// path are omitted, and unknown sections in user files are ignored.
// Generated once from that file; edit by hand.
#include "config.h"

namespace xmdg {
const std::string &defaults_yaml_text() {
    static const std::string text = R"XMDYAML(
general:
  total time: 20e3 tau
  seed: 42

langevin:
  enabled: true
  gamma factor: 2.0 1/tau
  temperature: 0.38 eps/kB

integrator:
  enabled: true
  dt: 5e-3 tau

neighbor list:
  pad factor: 0.25

tether forces:
  enabled: true
  H1: 100 eps/A**2
  H2: 0 eps/A**2
  default bond length: 3.8 A

native angles:
  enabled: true
  k: 30.0 eps/rad**2

complex native dihedrals:
  enabled: true
  CDA: 0.66 eps/rad**2
  CDB: 0.66 eps/rad**2

simple native dihedrals:
  enabled: false
  CDH: 3.33 eps/rad**2

heurestic angles:
  enabled: true
  coefficients: |-
    type1,type2,a0,a1,a2,a3,a4,a5
    G,G,20872.75597,-63260.52963,79318.301,-52680.17088,19554.21897,-3847.670279,313.6716916
    G,P,8222.83155,-25178.89003,31841.70634,-21290.04519,7941.501624,-1567.87285,128.0761621
    G,X,20872.75597,-63260.52963,79318.301,-52680.17088,19554.21897,-3847.670279,313.6716916
    P,G,34646.70029,-109957.2324,144423.9036,-100525.9874,39127.31928,-8079.214542,691.8417699
    P,P,10744.12043,-34148.94233,44818.66284,-31110.67875,12060.69185,-2479.723349,211.6367439
    P,X,34646.70029,-109957.2324,144423.9036,-100525.9874,39127.31928,-8079.214542,691.8417699
    X,G,15883.02041,-48923.1471,62360.6974,-42110.86572,15891.78309,-3178.490602,263.2916319
    X,P,16912.27207,-53570.09757,70150.19389,-48602.41198,18791.04978,-3844.690523,325.3085829
    X,X,15883.02041,-48923.1471,62360.6974,-42110.86572,15891.78309,-3178.490602,263.2916319

heurestic dihedrals:
  enabled: true
  coefficients: |-
    type2,type3,sin,cos,sin2,cos2,sin_cos
    G,G,0.133672207,-0.007576316,0.003786907,-0.124627339,0.425373566,-0.060606303,
    G,P,0.935285048,0.928786712,-0.18516837,0.015857805,0.2861951,0.072728001
    G,X,0.210489196,-0.00606094,0.202709724,-0.160512736,0.461339767,0.13333598
    P,G,0.233402207,-0.101516187,0.109235732,0.14906496,0.151803103,-0.742423775
    P,P,1.810497634,1.171212546,0.091084321,-0.254152251,0.557619284,-1.569694253
    P,X,0.661379307,0.115151794,0.428904959,0.200723546,0.100490651,-0.803028162
    X,P,0.198889776,0.018181703,-0.070746181,0.122076238,0.178719533,-0.624241103
    X,G,1.254229713,0.739393723,0.686217752,0.219188398,0.083115678,-0.790909154
    X,X,0.275933756,0.00606063,0.257226522,0.15460117,0.146208844,-0.448484074

native contacts:
  enabled: true
  lj depth: 1 eps
  active threshold: 1.5

chirality:
  enabled: false
  e_chi: 1 eps

native ssbonds:
  enabled: true
  H1: 100 eps/A**2
  equilibrium dist: 6.0 A

pseudo-improper dihedral potential:
  enabled: false
  lambda version: cosine
  bb+:
    alpha: 6.4 1/rad
    psi_0: 1.05 rad
    r_min: 5.6 A
    depth: 1 eps
  bb-:
    alpha: 6.0 1/rad
    psi_0: -1.44 rad
    r_min: 6.2 A
    depth: 1 eps
  ss:
    alpha: 1.2 1/rad
    psi_0: -0.23 rad

solid walls:
  enabled: false
  depth: 1 eps
  cutoff: 5.0 A

LJ attractive walls:
  enabled: false
  wall min dist: 5.0 A
  breaking factor: 1.5
  phase duration: 10 tau
  depth: 1 eps

velocity AFM:
  enabled: false
  H1: 0.06 eps/A**2
  H2: 0 eps/A**2

force AFM:
  enabled: false

Pauli exclusion:
  enabled: true
  r_excl: 4.0 A
  depth: 1.0 eps

const ES:
  enabled: true
  screening distance: 10.0 A
  permittivity: 80.0 eps_0

relative ES:
  enabled: false
  screening distance: 10.0 A
  factor: 4.0 eps_0/A

quasi-adiabatic potential:
  enabled: true
  phase duration: 10 tau
  breaking factor: 1.5
  min |cos(h, r)|: 0.92
  min |cos(h, h)| for bb: 0.75
  max cos(n, r): 0.5

lj force variants:
  bb:
    r_min: 5.0 A
    depth: 1.0 eps
  bs:
    r_min: 6.8 A
    depth: 1.0 eps
  ss:
    use sinking variant: true
    default:
      depth: 1.0 eps
    per pair:
      r_max: |-
        type,GLY,PRO,GLN,CYS,ALA,SER,VAL,THR,ILE,LEU,ASN,ASP,LYS,GLU,MET,HIS,PHE,ARG,TYR,TRP
        GLY,0,0,0,0,0,0,0,0,0,0,0,0,0,0,0,0,0,0,0,0
        PRO,0,7.41516,7.90612,7.52633,6.84509,7.04405,7.47655,7.31767,7.87539,8.01034,7.55152,7.23515,7.80572,7.53281,8.28535,7.90923,8.35495,8.6967,8.60035,8.73009
        GLN,0,7.90612,8.6339,7.72232,7.39072,7.63811,7.8121,7.76803,8.24492,8.43726,8.18851,8.15441,8.68554,8.40626,8.83875,8.64366,8.95351,9.25989,9.27035,9.58092
        CYS,0,7.52633,7.72232,7.55733,6.96894,6.97079,7.55818,7.4017,7.94719,8.07406,7.49217,7.17592,7.83117,7.44878,8.29132,8.1679,8.49679,8.24142,8.25576,8.94558
        ALA,0,6.84509,7.39072,6.96894,6.41596,6.52979,7.06164,6.94089,7.4515,7.64571,7.02481,6.73004,7.25636,7.03513,7.90635,7.49807,8.167,7.99254,8.01558,8.6489
        SER,0,7.04405,7.63811,6.97079,6.52979,6.64507,7.16628,6.96918,7.52021,7.68498,7.18018,6.99305,7.73488,7.40681,7.94113,7.87748,8.24345,8.27447,8.35846,8.753
        VAL,0,7.47655,7.8121,7.55818,7.06164,7.16628,7.64602,7.54035,8.06246,8.29202,7.53705,7.22267,7.68742,7.49567,8.48089,7.91666,8.68731,8.31488,8.38777,9.22171
        THR,0,7.31767,7.76803,7.4017,6.94089,6.96918,7.54035,7.30031,7.92881,8.12374,7.45743,7.19339,7.79424,7.50872,8.33046,7.97856,8.58396,8.49644,8.5783,9.13956
        ILE,0,7.87539,8.24492,7.94719,7.4515,7.52021,8.06246,7.92881,8.5263,8.77193,7.95509,7.65258,8.15891,7.97275,8.9472,8.36691,9.11118,8.75517,8.77521,9.57259
        LEU,0,8.01034,8.43726,8.07406,7.64571,7.68498,8.29202,8.12374,8.77193,8.93237,8.13966,7.85839,8.39261,8.19823,9.14397,8.56678,9.33507,8.98363,9.01661,9.78508
        ASN,0,7.55152,8.18851,7.49217,7.02481,7.18018,7.53705,7.45743,7.95509,8.13966,7.74478,7.49738,8.11461,7.99731,8.48918,8.36404,8.64859,8.87054,8.96106,9.10847
        ASP,0,7.23515,8.15441,7.17592,6.73004,6.99305,7.22267,7.19339,7.65258,7.85839,7.49738,7.3958,8.58582,7.81457,8.14884,8.49948,8.5134,9.12439,9.34604,9.10307
        LYS,0,7.80572,8.68554,7.83117,7.25636,7.73488,7.68742,7.79424,8.15891,8.39261,8.11461,8.58582,8.93192,8.90461,8.79787,8.57814,8.79341,9.49215,9.03734,9.20968
        GLU,0,7.53281,8.40626,7.44878,7.03513,7.40681,7.49567,7.50872,7.97275,8.19823,7.99731,7.81457,8.90461,8.37524,8.61045,8.8443,8.74517,9.51825,9.47761,9.47919
        MET,0,8.28535,8.83875,8.29132,7.90635,7.94113,8.48089,8.33046,8.9472,9.14397,8.48918,8.14884,8.79787,8.61045,9.29013,8.9267,9.55493,9.27252,9.28102,10.0219
        HIS,0,7.90923,8.64366,8.1679,7.49807,7.87748,7.91666,7.97856,8.36691,8.56678,8.36404,8.49948,8.57814,8.8443,8.9267,8.82674,8.97502,9.2293,9.38343,9.65746
        PHE,0,8.35495,8.95351,8.49679,8.167,8.24345,8.68731,8.58396,9.11118,9.33507,8.64859,8.5134,8.79341,8.74517,9.55493,8.97502,9.73068,9.2578,9.56181,10.168
        ARG,0,8.6967,9.25989,8.24142,7.99254,8.27447,8.31488,8.49644,8.75517,8.98363,8.87054,9.12439,9.49215,9.51825,9.27252,9.2293,9.2578,10.0222,9.50922,9.82199
        TYR,0,8.60035,9.27035,8.25576,8.01558,8.35846,8.38777,8.5783,8.77521,9.01661,8.96106,9.34604,9.03734,9.47761,9.28102,9.38343,9.56181,9.50922,9.34099,10.0829
        TRP,0,8.73009,9.58092,8.94558,8.6489,8.753,9.22171,9.13956,9.57259,9.78508,9.10847,9.10307,9.20968,9.47919,10.0219,9.65746,10.168,9.82199,10.0829,10.8456

amino acid data:
  amino acids:
    ALA:
      polarization: hydrophobic
      contact limits:
        back: 2
        side (all): 4
        side (hydrophobic): 1
        side (polar): 1
    ARG:
      polarization: polar
      charge: 1 e
      contact limits:
        back: 2
        side (all): 4
        side (hydrophobic): 0
        side (polar): 2
    ASN:
      polarization: polar
      contact limits:
        back: 2
        side (all): 3
        side (hydrophobic): 0
        side (polar): 2
    ASP:
      polarization: polar
      charge: -1 e
      contact limits:
        back: 2
        side (all): 2
        side (hydrophobic): 0
        side (polar): 2
    CYS:
      polarization: hydrophobic
      contact limits:
        back: 2
        side (all): 5
        side (hydrophobic): 2
        side (polar): 2
    GLU:
      polarization: polar
      charge: -1 e
      contact limits:
        back: 2
        side (all): 2
        side (hydrophobic): 0
        side (polar): 2
    GLN:
      polarization: polar
      contact limits:
        back: 2
        side (all): 3
        side (hydrophobic): 0
        side (polar): 2
    GLY:
      contact limits:
        back: 2
        side (all): 0
        side (hydrophobic): 0
        side (polar): 0
    HIS:
      polarization: polar
      contact limits:
        back: 2
        side (all): 4
        side (hydrophobic): 0
        side (polar): 2
    ILE:
      polarization: hydrophobic
      contact limits:
        back: 2
        side (all): 7
        side (hydrophobic): 4
        side (polar): 2
    LEU:
      polarization: hydrophobic
      contact limits:
        back: 2
        side (all): 7
        side (hydrophobic): 4
        side (polar): 2
    LYS:
      polarization: polar
      charge: 1 e
      contact limits:
        back: 2
        side (all): 3
        side (hydrophobic): 0
        side (polar): 2
    MET:
      polarization: hydrophobic
      contact limits:
        back: 2
        side (all): 7
        side (hydrophobic): 1
        side (polar): 1
    PHE:
      polarization: hydrophobic
      contact limits:
        back: 2
        side (all): 7
        side (hydrophobic): 4
        side (polar): 2
    PRO:
      contact limits:
        back: 1
        side (all): 0
        side (hydrophobic): 0
        side (polar): 0
    SER:
      polarization: polar
      contact limits:
        back: 2
        side (all): 2
        side (hydrophobic): 0
        side (polar): 2
    THR:
      polarization: polar
      contact limits:
        back: 2
        side (all): 3
        side (hydrophobic): 0
        side (polar): 2
    TRP:
      polarization: hydrophobic
      contact limits:
        back: 2
        side (all): 8
        side (hydrophobic): 4
        side (polar): 3
    TYR:
      polarization: hydrophobic
      contact limits:
        back: 2
        side (all): 7
        side (hydrophobic): 2
        side (polar): 2
    VAL:
      polarization: hydrophobic
      contact limits:
        back: 2
        side (all): 6
        side (hydrophobic): 4
        side (polar): 1

engine:
  precision: fp64
)XMDYAML";
    return text;
}
}  // namespace xmdg
