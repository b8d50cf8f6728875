"""Generates the golden fixtures of tests/golden/ by running the FargoCPT
reference itself.

Needs the reference sources (--ref=PATH or FARGO_REFERENCE_SRC: the
reference's src/ directory; by default a checkout named "reference" beside
the repository) and builds them with
oracle/ref/Makefile (parity flags: -O2 -fno-fast-math -ffp-contract=off) into
oracle/_ref/parity/fargocpt.  Each case writes a FargoCPT setup file plus a
seeded initial surface density (loaded by the reference via
``SigmaCondition: 2D``), runs the reference, and stores in <case>.npz:

* radii (Radii[0 .. Nrad+1]), the code-unit constants of constants.yml;
* the fields of snapshot 0 (initial state) and of the selected snapshots;
* the simulation time of every monitor output and the N-body positions and
  disk torques FargoCPT writes to monitor/nbody<k>.dat at each of them.

The generating setups are recorded next to the fixtures (<case>.yml) and the
engine parameters in <case>.json.  Run from the repository root:

    FARGO_REFERENCE_SRC=<reference>/src python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import json
import math
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from fargocpt_gb300.abi import ACCRETION, BC, COMPOSITE, DAMP, BETA_REF  # noqa: E402

# the reference's src/ directory: --ref=PATH, FARGO_REFERENCE_SRC, or a
# checkout named "reference" beside the repository
REF_SRC = os.environ.get("FARGO_REFERENCE_SRC",
                         os.path.join(os.path.dirname(REPO), "reference", "src"))
REF_EXE = os.path.join(REPO, "oracle", "_ref", "parity", "fargocpt")

COMMON = dict(
    l0="1 au", m0="1 solMass", mu=2.35, Sigma0=1e-3,
    ThicknessSmoothing=0.6, Integrator="Euler", InitializeVradialZero="yes",
    FirstDT=1.0, CFL=0.5, Frame="Fixed", HydroFrameCenter="primary",
    IndirectTermMode=1, DiskFeedback="no", RadialSpacing="Logarithmic",
    WriteDiskQuantities="no", Nmonitor=1,
)

# Each case: FargoCPT keys, grid, planet (or None), snapshots to keep.
CASES = {
    # C1-like: locally isothermal, one planet, SN art. visc, wave damping
    "iso_planet_fixed_dt": dict(
        keys=dict(SigmaSlope=0.5, AspectRatio=0.05, FlaringIndex=0.0,
                  EquationOfState="Isothermal", ViscousAlpha=1e-3,
                  ArtificialViscosity="SN", Transport="FARGO",
                  InnerBoundary="outflow", OuterBoundary="reference",
                  Damping="yes", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  DampingTimeFactor=1.0,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Reference",
                  DampingVAzimuthalOuter="Reference",
                  MonitorTimestep=0.002, Nsnapshots=20),
        nrad=20, naz=48, rmin=0.4, rmax=2.5, planet=1e-3, keep=[1, 2, 5, 10, 20]),
    # C2-like: adiabatic, beta cooling, SN with sqrt(2), flaring, planet
    "adi_planet_fixed_dt": dict(
        keys=dict(SigmaSlope=1.0, AspectRatio=0.05, FlaringIndex=0.25,
                  EquationOfState="Ideal", AdiabaticIndex=1.4, ViscousAlpha=1e-3,
                  ArtificialViscosity="SN", ArtificialViscosityFactor=1.41421356,
                  CoolingBetaLocal="yes", CoolingBeta=10,
                  Transport="FARGO",
                  InnerBoundary="zerogradient", OuterBoundary="outflow",
                  Damping="yes", DampingInnerLimit=1.15, DampingOuterLimit=0.85,
                  DampingTimeFactor=0.5,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Reference",
                  DampingVAzimuthalOuter="Reference",
                  DampingEnergyInner="Reference", DampingEnergyOuter="Reference",
                  MonitorTimestep=0.002, Nsnapshots=20),
        nrad=20, naz=48, rmin=0.3, rmax=3.0, planet=1e-3, keep=[1, 2, 5, 10, 20]),
    # CFL-limited, star only: exercises condition_cfl and the monitor clamp
    "iso_star_cfl": dict(
        keys=dict(SigmaSlope=0.5, AspectRatio=0.05, FlaringIndex=0.0,
                  EquationOfState="Isothermal", ViscousAlpha=1e-3,
                  ArtificialViscosity="SN", Transport="FARGO",
                  InnerBoundary="zerogradient", OuterBoundary="zerogradient",
                  Damping="yes", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Zero",
                  DampingVRadialInner="Zero", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Mean", DampingVAzimuthalOuter="Reference",
                  MonitorTimestep=0.5, Nsnapshots=4),
        nrad=16, naz=40, rmin=0.4, rmax=2.5, planet=None, keep=[1, 2, 3, 4]),
    # CFL-limited adiabatic, MC limiter, standard (non-FARGO) transport
    "adi_star_cfl_mc_std": dict(
        keys=dict(SigmaSlope=1.0, AspectRatio=0.05, FlaringIndex=0.25,
                  EquationOfState="Ideal", AdiabaticIndex=1.4, ViscousAlpha=3e-3,
                  ArtificialViscosity="SN", CoolingBetaLocal="yes", CoolingBeta=10,
                  FluxLimiter="mc", Transport="Standard",
                  InnerBoundary="outflow", OuterBoundary="zerogradient",
                  Damping="yes", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingEnergyInner="Mean", DampingEnergyOuter="Reference",
                  MonitorTimestep=0.05, Nsnapshots=3),
        nrad=16, naz=40, rmin=0.3, rmax=3.0, planet=None, keep=[1, 2, 3]),
    # LeapFrog (gas kick-drift-kick, simulation.cpp:276-459), locally
    # isothermal, CFL-limited, star only
    "iso_star_cfl_leapfrog": dict(
        keys=dict(SigmaSlope=0.5, AspectRatio=0.05, FlaringIndex=0.0,
                  EquationOfState="Isothermal", ViscousAlpha=1e-3,
                  ArtificialViscosity="SN", Transport="FARGO",
                  InnerBoundary="zerogradient", OuterBoundary="zerogradient",
                  Damping="yes", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Reference", DampingVAzimuthalOuter="Reference",
                  MonitorTimestep=0.5, Nsnapshots=4, Integrator="LeapFrog"),
        nrad=16, naz=40, rmin=0.4, rmax=2.5, planet=None, keep=[1, 2, 3, 4]),
    # LeapFrog, adiabatic with beta cooling and SN, FARGO, star only
    "adi_star_cfl_leapfrog": dict(
        keys=dict(SigmaSlope=1.0, AspectRatio=0.05, FlaringIndex=0.25,
                  EquationOfState="Ideal", AdiabaticIndex=1.4, ViscousAlpha=1e-3,
                  ArtificialViscosity="SN", ArtificialViscosityFactor=1.41421356,
                  CoolingBetaLocal="yes", CoolingBeta=10, Transport="FARGO",
                  InnerBoundary="zerogradient", OuterBoundary="outflow",
                  Damping="yes", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Reference", DampingVAzimuthalOuter="Reference",
                  DampingEnergyInner="Reference", DampingEnergyOuter="Reference",
                  MonitorTimestep=0.4, Nsnapshots=4, Integrator="LeapFrog"),
        nrad=16, naz=40, rmin=0.3, rmax=3.0, planet=None, keep=[1, 2, 3, 4]),
    # Tscharnuter-Winkler artificial viscosity, adiabatic, planet, fixed dt
    "adi_planet_tw": dict(
        keys=dict(SigmaSlope=1.0, AspectRatio=0.05, FlaringIndex=0.25,
                  EquationOfState="Ideal", AdiabaticIndex=1.4, ViscousAlpha=3e-2,
                  ArtificialViscosity="TW", ArtificialViscosityFactor=1.41421356,
                  CoolingBetaLocal="yes", CoolingBeta=10,
                  Transport="FARGO",
                  InnerBoundary="zerogradient", OuterBoundary="outflow",
                  Damping="yes", DampingInnerLimit=1.15, DampingOuterLimit=0.85,
                  DampingTimeFactor=0.5,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Reference",
                  DampingVAzimuthalOuter="Reference",
                  DampingEnergyInner="Reference", DampingEnergyOuter="Reference",
                  MonitorTimestep=0.002, Nsnapshots=20),
        nrad=20, naz=48, rmin=0.3, rmax=3.0, planet=1e-3, keep=[1, 2, 5, 10, 20]),
    # TW with the pseudo-implicit viscous update (StabilizeViscosity 1):
    # viscosity-dominated CFL at CFL 1.3, so that dt |c| exceeds 1 in cells
    # and the correction acts; adiabatic, star only
    "adi_star_cfl_tw_stab1": dict(
        keys=dict(SigmaSlope=1.0, AspectRatio=0.05, FlaringIndex=0.25,
                  EquationOfState="Ideal", AdiabaticIndex=1.4, ConstantViscosity=1e-2,
                  ArtificialViscosity="TW", StabilizeViscosity=1, CFL=1.3,
                  CoolingBetaLocal="yes", CoolingBeta=10, Transport="FARGO",
                  InnerBoundary="zerogradient", OuterBoundary="zerogradient",
                  Damping="yes", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Reference", DampingVAzimuthalOuter="Reference",
                  DampingEnergyInner="Reference", DampingEnergyOuter="Reference",
                  MonitorTimestep=0.3, Nsnapshots=3),
        nrad=16, naz=40, rmin=0.4, rmax=2.5, planet=None, keep=[1, 2, 3]),
    # Accretion onto the planet (accretion.cpp:84-480), Kley's two zones,
    # locally isothermal, fixed dt; the planet's mass stays fixed
    # (DiskFeedback no), the accreted mass is in the monitor's accretion rate
    "iso_planet_accretion_kley": dict(
        keys=dict(SigmaSlope=0.5, AspectRatio=0.05, FlaringIndex=0.0,
                  EquationOfState="Isothermal", ViscousAlpha=1e-3,
                  ArtificialViscosity="SN", Transport="FARGO",
                  InnerBoundary="outflow", OuterBoundary="reference",
                  Damping="yes", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Reference",
                  DampingVAzimuthalOuter="Reference",
                  MassAccretionRadius=2.0, MonitorTimestep=0.002, Nsnapshots=20),
        nrad=24, naz=64, rmin=0.4, rmax=2.5, planet=3e-3,
        planet_keys={"accretion efficiency": 10, "accretion method": "kley"},
        keep=[1, 2, 5, 10, 20]),
    # sink-hole accretion, adiabatic
    "adi_planet_accretion_sinkhole": dict(
        keys=dict(SigmaSlope=1.0, AspectRatio=0.05, FlaringIndex=0.25,
                  EquationOfState="Ideal", AdiabaticIndex=1.4, ViscousAlpha=1e-3,
                  ArtificialViscosity="SN", ArtificialViscosityFactor=1.41421356,
                  CoolingBetaLocal="yes", CoolingBeta=10, Transport="FARGO",
                  InnerBoundary="zerogradient", OuterBoundary="outflow",
                  Damping="yes", DampingInnerLimit=1.15, DampingOuterLimit=0.85,
                  DampingTimeFactor=0.5,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Reference",
                  DampingVAzimuthalOuter="Reference",
                  DampingEnergyInner="Reference", DampingEnergyOuter="Reference",
                  MassAccretionRadius=1.5, MonitorTimestep=0.002, Nsnapshots=20),
        nrad=24, naz=64, rmin=0.3, rmax=3.0, planet=3e-3,
        planet_keys={"accretion efficiency": 5, "accretion method": "sinkhole"},
        keep=[1, 2, 5, 10, 20]),
    # viscous accretion profile (M_dot = 3 pi nu Sigma), locally isothermal
    "iso_planet_accretion_viscous": dict(
        keys=dict(SigmaSlope=0.5, AspectRatio=0.05, FlaringIndex=0.0,
                  EquationOfState="Isothermal", ViscousAlpha=1e-2,
                  ArtificialViscosity="SN", Transport="FARGO",
                  InnerBoundary="outflow", OuterBoundary="reference",
                  Damping="yes", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Reference",
                  DampingVAzimuthalOuter="Reference",
                  MassAccretionRadius=2.0, MonitorTimestep=0.002, Nsnapshots=20),
        nrad=24, naz=64, rmin=0.4, rmax=2.5, planet=3e-3,
        planet_keys={"accretion efficiency": 300, "accretion method": "viscous"},
        keep=[1, 2, 5, 10, 20]),
    # per-field boundary hooks: disk model, reflecting, zero shear, Keplerian
    # radial, balanced; locally isothermal, planet, fixed dt, no damping
    "iso_planet_bc_individual": dict(
        keys=dict(SigmaSlope=0.5, AspectRatio=0.05, FlaringIndex=0.0,
                  EquationOfState="Isothermal", ViscousAlpha=1e-3,
                  ArtificialViscosity="SN", Transport="FARGO",
                  InnerBoundary="individual", OuterBoundary="individual",
                  InnerBoundarySigma="diskmodel", InnerBoundaryEnergy="zerogradient",
                  InnerBoundaryVrad="reflecting", InnerBoundaryVazi="zeroshear",
                  OuterBoundarySigma="zerogradient", OuterBoundaryEnergy="zerogradient",
                  OuterBoundaryVrad="keplerian", OuterBoundaryVradKeplerianFactor=0.05,
                  OuterBoundaryVazi="balanced",
                  Damping="no", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  MonitorTimestep=0.002, Nsnapshots=20),
        nrad=20, naz=48, rmin=0.4, rmax=2.5, planet=1e-3, keep=[1, 2, 5, 10, 20]),
    # viscous outflow at the inner edge, balanced inner, zero-shear outer,
    # disk-model sigma and energy; adiabatic, CFL-limited, damping on
    "adi_star_cfl_bc_individual": dict(
        keys=dict(SigmaSlope=1.0, AspectRatio=0.05, FlaringIndex=0.25,
                  EquationOfState="Ideal", AdiabaticIndex=1.4, ViscousAlpha=1e-2,
                  ArtificialViscosity="SN", CoolingBetaLocal="yes", CoolingBeta=10,
                  Transport="FARGO",
                  InnerBoundary="individual", OuterBoundary="individual",
                  InnerBoundarySigma="reference", InnerBoundaryEnergy="diskmodel",
                  InnerBoundaryVrad="viscous", InnerBoundaryVazi="balanced",
                  OuterBoundarySigma="diskmodel", OuterBoundaryEnergy="diskmodel",
                  OuterBoundaryVrad="reflecting", OuterBoundaryVazi="zeroshear",
                  ViscousOutflowSpeed=2.0,
                  Damping="yes", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingEnergyInner="Reference", DampingEnergyOuter="Reference",
                  MonitorTimestep=0.4, Nsnapshots=4),
        nrad=16, naz=40, rmin=0.3, rmax=3.0, planet=None, keep=[1, 2, 3, 4]),
    # TW with the viscous stability dt limit (StabilizeViscosity 2), locally
    # isothermal, a viscosity-dominated CFL so that the limit binds
    "iso_star_cfl_tw_stab2": dict(
        keys=dict(SigmaSlope=0.5, AspectRatio=0.05, FlaringIndex=0.0,
                  EquationOfState="Isothermal", ConstantViscosity=1e-2,
                  ArtificialViscosity="TW", StabilizeViscosity=2, Transport="FARGO",
                  InnerBoundary="zerogradient", OuterBoundary="zerogradient",
                  Damping="yes", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Reference", DampingVAzimuthalOuter="Reference",
                  MonitorTimestep=0.05, Nsnapshots=4),
        nrad=16, naz=40, rmin=0.4, rmax=2.5, planet=None, keep=[1, 2, 3, 4]),
    # centre-of-mass composite at both edges (center_of_mass.cpp) with its
    # damping: locally isothermal, one planet (the star-planet pair takes the
    # binary branch of the viscous-speed tables), fixed dt
    "iso_planet_bc_com": dict(
        keys=dict(SigmaSlope=0.5, AspectRatio=0.05, FlaringIndex=0.0,
                  EquationOfState="Isothermal", ViscousAlpha=1e-3,
                  ArtificialViscosity="SN", Transport="FARGO",
                  InnerBoundary="centerofmass", OuterBoundary="centerofmass",
                  Damping="yes", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  MonitorTimestep=0.002, Nsnapshots=20),
        nrad=20, naz=48, rmin=0.4, rmax=2.5, planet=1e-3, keep=[1, 2, 5, 10, 20]),
    # corotating frame (refframe::handle_corotation): OmegaFrame follows the
    # planet, v_phi corrected by its change every step; locally isothermal,
    # fixed dt, damping, outflow / reference edges
    "iso_planet_corotating": dict(
        keys=dict(SigmaSlope=0.5, AspectRatio=0.05, FlaringIndex=0.0,
                  EquationOfState="Isothermal", ViscousAlpha=1e-3,
                  ArtificialViscosity="SN", Transport="FARGO", Frame="Corotating",
                  InnerBoundary="outflow", OuterBoundary="reference",
                  Damping="yes", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Reference", DampingVAzimuthalOuter="Reference",
                  MonitorTimestep=0.002, Nsnapshots=20),
        nrad=20, naz=48, rmin=0.4, rmax=2.5, planet=1e-3, keep=[1, 2, 5, 10, 20]),
    # the same with the Keplerian model (InitializePureKeplerian): adiabatic,
    # star only, CFL-limited, energy damping
    "adi_star_cfl_bc_com_keplerian": dict(
        keys=dict(SigmaSlope=1.0, AspectRatio=0.05, FlaringIndex=0.25,
                  EquationOfState="Ideal", AdiabaticIndex=1.4, ViscousAlpha=1e-2,
                  ArtificialViscosity="SN", CoolingBetaLocal="yes", CoolingBeta=10,
                  Transport="FARGO", InitializePureKeplerian="yes",
                  InnerBoundary="centerofmass", OuterBoundary="centerofmass",
                  Damping="yes", DampingInnerLimit=1.2, DampingOuterLimit=0.85,
                  MonitorTimestep=0.4, Nsnapshots=4),
        nrad=16, naz=40, rmin=0.3, rmax=3.0, planet=None, keep=[1, 2, 3, 4]),
    # the viscous-speed model at an adiabatic disk with a planet: the outer
    # grid correction of the tables, energy at both ghost rings
    "adi_planet_bc_com": dict(
        keys=dict(SigmaSlope=1.0, AspectRatio=0.05, FlaringIndex=0.25,
                  EquationOfState="Ideal", AdiabaticIndex=1.4, ViscousAlpha=3e-3,
                  ArtificialViscosity="SN", CoolingBetaLocal="yes", CoolingBeta=10,
                  Transport="FARGO",
                  InnerBoundary="zerogradient", OuterBoundary="centerofmass",
                  Damping="yes", DampingInnerLimit=1.15, DampingOuterLimit=0.85,
                  DampingSurfaceDensityInner="Reference",
                  DampingVRadialInner="Reference", DampingVAzimuthalInner="Reference",
                  DampingEnergyInner="Reference",
                  MonitorTimestep=0.002, Nsnapshots=20),
        nrad=20, naz=48, rmin=0.3, rmax=3.0, planet=3e-3, keep=[1, 2, 5, 10, 20]),
    # KeepDiskMassConstant (sigma rescaled after every final boundary call,
    # simulation.cpp:246-251), CorrectDiskSelfgravity off (the disk force from
    # sigma itself, Force.cpp:64-66), and the monitor quantities
    # (Quantities.dat: mass and angular momentum within QuantitiesRadiusLimit,
    # output.cpp:326-470) for gas_total_mass / gas_angular_momentum
    "adi_planet_keep_mass_nocorr": dict(
        keys=dict(SigmaSlope=1.0, AspectRatio=0.05, FlaringIndex=0.25,
                  EquationOfState="Ideal", AdiabaticIndex=1.4, ViscousAlpha=1e-3,
                  ArtificialViscosity="SN", ArtificialViscosityFactor=1.41421356,
                  CoolingBetaLocal="yes", CoolingBeta=10,
                  Transport="FARGO",
                  InnerBoundary="outflow", OuterBoundary="outflow",
                  Damping="yes", DampingInnerLimit=1.15, DampingOuterLimit=0.85,
                  DampingTimeFactor=0.5,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Reference",
                  DampingVAzimuthalOuter="Reference",
                  DampingEnergyInner="Reference", DampingEnergyOuter="Reference",
                  KeepDiskMassConstant="yes", CorrectDiskSelfgravity="no",
                  WriteDiskQuantities="yes", QuantitiesRadiusLimit=1.5,
                  MonitorTimestep=0.002, Nsnapshots=20),
        nrad=20, naz=48, rmin=0.3, rmax=3.0, planet=1e-3, keep=[1, 2, 5, 10, 20]),
    # The locally isothermal 128 x 384 disk with one planet of the benchmark
    # set (FARGO, reference damping at both edges, CFL 0.5) over about a
    # hundred CFL-limited steps; the planet moves on its circular orbit
    # between the monitor outputs, so the replay takes its position from the
    # orbit (circular_bodies) at every step.
    "c1_cfl_100": dict(
        keys=dict(SigmaSlope=0.5, AspectRatio=0.05, FlaringIndex=0.0,
                  EquationOfState="Isothermal", ViscousAlpha=1e-3,
                  ArtificialViscosity="SN", Transport="FARGO",
                  InnerBoundary="reference", OuterBoundary="reference",
                  Damping="yes", DampingInnerLimit=1.1, DampingOuterLimit=0.9,
                  DampingTimeFactor=1.0,
                  DampingSurfaceDensityInner="Reference",
                  DampingSurfaceDensityOuter="Reference",
                  DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
                  DampingVAzimuthalInner="Reference",
                  DampingVAzimuthalOuter="Reference",
                  MonitorTimestep=0.2, Nsnapshots=10),
        nrad=128, naz=384, rmin=0.4, rmax=2.5, planet=1e-3, keep=[10],
        circular_bodies=True),
}


def build_reference():
    if not REF_SRC or not os.path.isdir(REF_SRC):
        raise SystemExit("set FARGO_REFERENCE_SRC (or --ref=PATH) to the reference's src/ "
                         f"directory (got {REF_SRC!r})")
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle", "ref"),
                    "VARIANT=parity", f"REF={REF_SRC}", "-j8"], check=True)


def log_radii(nrad, rmin, rmax):
    q = math.pow(rmax / rmin, 1.0 / (nrad - 2.0))
    return np.array([rmin * math.pow(q, n - 1.0) for n in range(nrad + 2)])


def read_yaml_values(path):
    """Tiny reader for FargoCPT's constants.yml / units.yml blocks."""
    out, cur = {}, None
    for line in open(path):
        if not line.strip() or line.startswith("#"):
            continue
        if not line.startswith(" "):
            cur = line.strip().rstrip(":")
            out[cur] = {}
        else:
            k, _, v = line.strip().partition(":")
            out[cur][k.strip()] = v.strip()
    return out


def engine_params(case, consts, temp_unit):
    k = {**COMMON, **case["keys"]}
    adi = k["EquationOfState"].lower() in ("ideal", "adiabatic")
    inner, outer = k["InnerBoundary"].lower(), k["OuterBoundary"].lower()

    def composite(name):   # boundary_conditions/config.cpp:344-430
        return {"zerogradient": ("zerogradient", "zerogradient", "zerogradient"),
                "outflow": ("zerogradient", "zerogradient", "outflow"),
                "reference": ("reference", "reference", "reference"),
                "centerofmass": ("none", "none", "none")}[name]

    def side_names(side, comp):
        # per-field names after the composite and the individual keys
        # (config.cpp:75-96, 345-440); the inner energy hook reads and
        # overwrites the outer name (config.cpp:147)
        names = dict(zip(("sigma", "energy", "vrad"),
                         composite(comp) if comp != "individual" else ("", "", "")))
        for key, fld in (("Sigma", "sigma"), ("Vrad", "vrad")):
            if f"{side}Boundary{key}" in k:
                names[fld] = str(k[f"{side}Boundary{key}"]).lower()
        default_vazi = "none" if comp == "centerofmass" else "keplerian"
        names["vazi"] = str(k.get(f"{side}BoundaryVazi", default_vazi)).lower()
        return names

    nin, nout = side_names("Inner", inner), side_names("Outer", outer)
    energy_outer_name = nout["energy"]
    if "InnerBoundaryEnergy" in k:
        energy_outer_name = str(k["InnerBoundaryEnergy"]).lower()
    ei = energy_outer_name
    eo = str(k.get("OuterBoundaryEnergy", energy_outer_name)).lower()
    si, vi, so, vo = nin["sigma"], nin["vrad"], nout["sigma"], nout["vrad"]

    def vrad_kind(name):
        return BC["keplerian_radial"] if name == "keplerian" else BC[name]

    def damp(key):
        v = str(k.get(key, "None")).lower()[0]
        return {"n": 0, "r": 1, "i": 1, "y": 1, "m": 3, "z": 2}[v]

    return dict(
        nrad=case["nrad"], naz=case["naz"], eos=1 if adi else 0,
        art_visc={"s": 1, "t": 2, "n": 0}[str(k.get("ArtificialViscosity", "SN")).lower()[0]],
        stabilize_viscosity=int(k.get("StabilizeViscosity", 0)),
        art_visc_dissipation=1, flux_limiter=1 if k.get("FluxLimiter", "") == "mc" else 0,
        fast_transport=1 if k["Transport"].lower().startswith("f") else 0,
        heating_viscous=1, cooling_beta=1 if k.get("CoolingBetaLocal") == "yes" else 0,
        cooling_beta_reference=BETA_REF["zero"],
        damping=int(str(k.get("Damping", "no")).lower() in ("yes", "true", "1")),
        damping_inner=[damp("DampingVRadialInner"), damp("DampingVAzimuthalInner"),
                       damp("DampingSurfaceDensityInner"), damp("DampingEnergyInner")],
        damping_outer=[damp("DampingVRadialOuter"), damp("DampingVAzimuthalOuter"),
                       damp("DampingSurfaceDensityOuter"), damp("DampingEnergyOuter")],
        bc_sigma_inner=BC[si], bc_sigma_outer=BC[so],
        bc_energy_inner=BC[ei], bc_energy_outer=BC[eo],
        bc_vrad_inner=vrad_kind(vi), bc_vrad_outer=vrad_kind(vo),
        bc_vaz_inner=BC[nin["vazi"]], bc_vaz_outer=BC[nout["vazi"]],
        sigma_slope=float(k["SigmaSlope"]),
        viscous_outflow_speed=float(k.get("ViscousOutflowSpeed", 1.0)),
        vrad_inner_keplerian_factor=float(k.get("InnerBoundaryVradKeplerianFactor", 0.1)),
        vrad_outer_keplerian_factor=float(k.get("OuterBoundaryVradKeplerianFactor", 0.1)),
        precision=0,
        accretion_radius_fraction=float(k.get("MassAccretionRadius", 1.0)),
        integrator=1 if str(k.get("Integrator", "Euler")).lower().startswith("l") else 0,
        gamma=float(k.get("AdiabaticIndex", 1.4)), mu=float(k["mu"]),
        aspect_ratio=float(k["AspectRatio"]), flaring_index=float(k["FlaringIndex"]),
        viscous_alpha=float(k.get("ViscousAlpha", 0.0)),
        constant_viscosity=float(k.get("ConstantViscosity", 0.0)),
        art_visc_factor=float(k.get("ArtificialViscosityFactor", 1.41)),
        radial_viscosity_factor=1.0, heating_viscous_factor=1.0,
        cfl=float(k["CFL"]), cfl_max_var=1.1, heating_cooling_cfl_limit=10.0,
        sigma0=float(k["Sigma0"]), sigma_floor=1e-9,
        thickness_smoothing=float(k["ThicknessSmoothing"]),
        cooling_beta_value=float(k.get("CoolingBeta", 1.0)), cooling_beta_ramp_up=0.0,
        minimum_temperature=3.0 / temp_unit, maximum_temperature=1.0e300 / temp_unit,
        G=float(consts["gravitational constant"]["code value"]),
        R_gas=float(consts["specific gas constant"]["code value"]),
        sigma_sb=float(consts["Stefan-Boltzmann constant"]["code value"]),
        c_light=float(consts["speed of light"]["code value"]),
        hydro_center_mass=1.0,
        damping_inner_limit=float(k["DampingInnerLimit"]),
        damping_outer_limit=float(k["DampingOuterLimit"]),
        damping_time_factor=float(k.get("DampingTimeFactor", 1.0)),
        damping_time_radius_outer=float(case["rmax"]),
        vaz_inner_keplerian_factor=1.0, vaz_outer_keplerian_factor=1.0,
        rmin=float(case["rmin"]), rmax=float(case["rmax"]), radial_spacing=1,
        composite_inner=COMPOSITE.get(inner, 0), composite_outer=COMPOSITE.get(outer, 0),
        initialize_pure_keplerian=int(str(k.get("InitializePureKeplerian", "no")) == "yes"),
        initialize_vradial_zero=int(str(k.get("InitializeVradialZero", "no")) == "yes"),
        profile_cutoff_point_outer=1.0e300, profile_cutoff_width_outer=1.0,
        profile_cutoff_point_inner=0.0, profile_cutoff_width_inner=1.0,
        temperature_cgs_to_code=1.0 / temp_unit,
        # parameters::VISCOUS_ACCRETION: a planet accreting with the viscous
        # profile or the viscous v_radial hook (planetary_system.cpp:255-257,
        # Interpret.cpp:704-707)
        viscous_accretion=int(str(case.get("planet_keys", {}).get("accretion method", ""))
                              == "viscous" or vi == "viscous" or vo == "viscous"),
        keep_disk_mass_constant=int(str(k.get("KeepDiskMassConstant", "no")) == "yes"),
        correct_disk_selfgravity=int(str(k.get("CorrectDiskSelfgravity", "yes")) == "yes"),
    )


def write_setup(case, path, seed):
    nrad, naz = case["nrad"], case["naz"]
    radii = log_radii(nrad, case["rmin"], case["rmax"])
    rinf, rsup = radii[:nrad], radii[1:nrad + 1]
    rmed = 2.0 / 3.0 * (rsup ** 3 - rinf ** 3) / (rsup ** 2 - rinf ** 2)
    rng = np.random.default_rng(seed)
    slope = case["keys"]["SigmaSlope"]
    sigma = 1e-3 * rmed[:, None] ** -slope * (1 + 1e-3 * rng.uniform(-1, 1, (nrad, naz)))
    sigma.astype("<f8").tofile(os.path.join(path, "sigma_init.dat"))
    keys = {**COMMON, **case["keys"], "Nrad": nrad, "Naz": naz,
            "Rmin": case["rmin"], "Rmax": case["rmax"],
            "SigmaCondition": "2D", "SigmaFilename": "sigma_init.dat",
            "OutputDir": "out"}
    lines = [f"{k}: {v}" for k, v in keys.items()]
    lines.append("nbody:")
    lines.append("- name: star\n  semi-major axis: 0.0\n  mass: 1.0")
    if case["planet"] is not None:
        lines.append(f"- name: planet\n  semi-major axis: 1.0\n  mass: {case['planet']}\n"
                     "  eccentricity: 0.0")
        for key, v in case.get("planet_keys", {}).items():
            lines.append(f"  {key}: {v}")
    text = "\n".join(lines) + "\n"
    with open(os.path.join(path, "setup.yml"), "w") as f:
        f.write(text)
    return text


def read_snapshot(out, n, nrad, naz):
    d = os.path.join(out, "snapshots", str(n))

    def rd(name, rows):
        return np.fromfile(os.path.join(d, name), dtype="<f8").reshape(rows, naz)

    return dict(SIGMA=rd("Sigma.dat", nrad), V_RADIAL=rd("vrad.dat", nrad + 1),
                V_AZIMUTHAL=rd("vazi.dat", nrad), ENERGY=rd("energy.dat", nrad))


def read_nbody(out, k):
    rows = []
    for line in open(os.path.join(out, "monitor", f"nbody{k}.dat")):
        if line.startswith("#") or not line.strip():
            continue
        rows.append([float(x) for x in line.split()])
    a = np.array(rows)
    # columns (nbody/planet.cpp:361-372): snapshot, monitor, x, y, vx, vy,
    # mass, time, omega_frame, ..., torque (18), accretion torque (19),
    # indirect torque (20), accretion rate (21)
    return dict(x=a[:, 2], y=a[:, 3], vx=a[:, 4], vy=a[:, 5], mass=a[:, 6], time=a[:, 7],
                omega_frame=a[:, 8], torque=a[:, 18], accretion_rate=a[:, 21])


def read_quantities(out):
    """monitor/Quantities.dat (output.cpp:326-470): per monitor row the
    monitor number, time, gas mass and angular momentum within
    QuantitiesRadiusLimit."""
    rows = []
    for line in open(os.path.join(out, "monitor", "Quantities.dat")):
        if line.startswith("#") or not line.strip():
            continue
        v = line.split()
        rows.append([float(v[1]), float(v[2]), float(v[3]), float(v[5])])
    a = np.array(rows)
    return dict(monitor=a[:, 0].astype(np.int64), time=a[:, 1], mass=a[:, 2],
                angular_momentum=a[:, 3])


def make_case(name, case, seed):
    tmp = tempfile.mkdtemp(prefix=f"golden_{name}_")
    try:
        text = write_setup(case, tmp, seed)
        r = subprocess.run([REF_EXE, "start", "setup.yml"], cwd=tmp,
                           capture_output=True, text=True, timeout=600,
                           env={**os.environ, "OMP_NUM_THREADS": "1"})
        if r.returncode != 0:
            print(r.stdout[-3000:], r.stderr[-3000:])
            raise SystemExit(f"reference run {name} failed")
        out = os.path.join(tmp, "out")
        nrad, naz = case["nrad"], case["naz"]
        used = np.loadtxt(os.path.join(out, "used_rad.dat"))
        radii = log_radii(nrad, case["rmin"], case["rmax"])
        assert np.array_equal(used, radii[:nrad + 1]), "radii formula mismatch"
        consts = read_yaml_values(os.path.join(out, "constants.yml"))
        units = read_yaml_values(os.path.join(out, "units.yml"))
        temp_unit = float(units["temperature"]["cgs value"])
        params = engine_params(case, consts, temp_unit)
        arrays = {"radii": radii}
        snap0 = read_snapshot(out, 0, nrad, naz)
        for k, v in snap0.items():
            arrays[f"s0_{k}"] = v
        for n in case["keep"]:
            for k, v in read_snapshot(out, n, nrad, naz).items():
                arrays[f"s{n}_{k}"] = v
            # the snapshot's misc.bin as written (struct misc_entry,
            # output.h:14-22, output.cpp:494-527), byte for byte
            with open(os.path.join(out, "snapshots", str(n), "misc.bin"), "rb") as f:
                arrays[f"s{n}_misc"] = np.frombuffer(f.read(), dtype=np.uint8)
        nb = 2 if case["planet"] is not None else 1
        for k in range(nb):
            for key, v in read_nbody(out, k).items():
                arrays[f"body{k}_{key}"] = v
        arrays["keep"] = np.array(case["keep"])
        if str(case["keys"].get("WriteDiskQuantities", "no")) == "yes":
            for key, v in read_quantities(out).items():
                arrays[f"quantities_{key}"] = v
        meta = dict(params=params, first_dt=float(COMMON["FirstDT"]),
                    monitor_timestep=float(case["keys"]["MonitorTimestep"]),
                    nsnapshots=int(case["keys"]["Nsnapshots"]), nbodies=nb,
                    seed=seed, reference_log_tail=r.stdout.splitlines()[-1])
        if str(case["keys"].get("Frame", COMMON["Frame"])).lower().startswith("c"):
            meta["corotating"] = True
        if case.get("circular_bodies"):
            meta["circular_bodies"] = True
        if "QuantitiesRadiusLimit" in case["keys"]:
            meta["quantities_radius"] = float(case["keys"]["QuantitiesRadiusLimit"])
        if case.get("planet_keys"):
            pk = case["planet_keys"]
            meta["accretion"] = dict(type=ACCRETION[pk["accretion method"]],
                                     efficiency=float(pk["accretion efficiency"]))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
        with open(os.path.join(HERE, f"{name}.json"), "w") as f:
            json.dump(meta, f, indent=1, sort_keys=True)
        with open(os.path.join(HERE, f"{name}.yml"), "w") as f:
            f.write("# FargoCPT setup that produced the fixture (sigma file: seeded noise)\n")
            f.write(text)
        print(f"{name}: ok ({meta['reference_log_tail']})")
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def main():
    """python make_golden.py [--ref=PATH] [case ...]: all cases, or the named ones."""
    global REF_SRC
    args = []
    for a in sys.argv[1:]:
        if a.startswith("--ref="):
            REF_SRC = a[len("--ref="):]
        else:
            args.append(a)
    build_reference()
    only = set(args)
    for i, (name, case) in enumerate(CASES.items()):
        if only and name not in only:
            continue
        # a fixture keeps the seed it was first made with
        seed = 1000 + i
        meta_path = os.path.join(HERE, f"{name}.json")
        if os.path.exists(meta_path):
            with open(meta_path) as f:
                seed = int(json.load(f).get("seed", seed))
        make_case(name, case, seed=seed)


if __name__ == "__main__":
    main()
