"""The workloads the solver is measured and checked on, built through the reference API.

Each builder takes the solver class to instantiate (so the same scene can be run on the GPU
and through the CPU oracle) and returns ``(solver, mesh, info)``.

* ``taylor_rod``   -- the axisymmetric Taylor impact: TaylorImpactCase.run
                     (validate/TaylorImpactCase.java:214-331), and the 10 x 60 rod used as the
                     plain FP64 parity case;
* ``perforation``  -- the plane-strain multi-body scene: a steel slug through a stacked wall of
                     copper blocks on a rigid floor, the template of Smash.main (Smash.java:82-150)
                     at the sizes of the 200k-quad perforation benchmark;
* ``two_blocks``   -- Bench.build (Bench.java:142-169): two copper bodies, optional damage,
                     floor and contact;
* ``tube``         -- the pressurised thin wall of DefectBurst.fire / BurstCase.run
                     (QuadMesh.cylinderWall, smoothstep pressure ramp, relaxation damping);
* ``taylor_sweep`` -- a sweep of Taylor rods with drawn meshes, Johnson-Cook constants,
                     friction and speeds (the batched workload; Sweep.over over
                     TaylorImpactCase.run).
"""
from __future__ import annotations

import math

import numpy as np

from .defects import DefectField, Weibull
from .materials import Formulation, Integration, JohnsonCook, Kinematics, Material, Materials
from .mesh import Outline, QuadMesh
from .solver import Contact, RigidWall

MM = 1.0e-3

# The 10 x 60 rod's steel: E 200 GPa, nu 0.29, rho 7850, Johnson-Cook (350 MPa, 275 MPa,
# 0.36, 0.022, m 1.0, 1/s, 293 K, 1793 K, 477 J/kgK, 0.9).
ROD_JC = JohnsonCook(350.0e6, 275.0e6, 0.36, 0.022, 1.0, 1.0, 293.0, 1793.0, 477.0, 0.9)
# Kinematic fraction 0.3 of the Johnson-Cook secant modulus at 0.6 plastic strain (the fit
# strain the reference's rate-independent surrogate uses, TaylorImpactCase.java:147-152).
ROD_KINEMATIC_FRACTION = 0.3
ROD_FIT_STRAIN = 0.6


def rod_material() -> Material:
    secant = ROD_JC.b * ROD_FIT_STRAIN ** ROD_JC.n / ROD_FIT_STRAIN
    base = Material("rod steel", 200.0e9, 0.29, 7850.0)
    return base.withKinematicHardening(ROD_KINEMATIC_FRACTION * secant).withJohnsonCook(ROD_JC)


def taylor_rod(cls, nr=10, nz=60, radius=3.8e-3, length=25.0e-3, speed=200.0, friction=0.09,
               cfl=0.6, hourglass=0.10, integration=Integration.REDUCED, material=None):
    """The axisymmetric rod on a rigid Coulomb anvil (TaylorImpactCase.java:214-258)."""
    mesh = QuadMesh.solidCylinder(radius, length, nr, nz)
    mat = material if material is not None else rod_material()
    s = cls(mesh, mat, Formulation.AXISYMMETRIC, integration, Kinematics.FINITE_STRAIN, 1.0, cfl)
    s.setHourglassCoefficient(hourglass)
    for n in QuadMesh.axisNodes(nr, nz):
        s.fixRadial(n)
    wall = RigidWall.atZ(0.0, friction)
    s.setRigidWall(wall)
    s.setUniformVelocity(0.0, -speed)
    return s, mesh, {"wall": wall, "length": length}


def taylor_reference(cls, nr, integration=Integration.REDUCED, friction=0.0, jc=True):
    """TaylorImpactCase.referenceAt: 4340 steel, 37.97 x 7.595 mm, 181 m/s, square cells."""
    L, D = 37.97e-3, 7.595e-3
    R = 0.5 * D
    h = R / nr
    nz = max(1, int(math.floor(L / h + 0.5)))
    if jc:
        mat = Material.STEEL_4340.withJohnsonCook(JohnsonCook.STEEL_4340)
    else:
        jc4340 = JohnsonCook.STEEL_4340
        secant = jc4340.b * 0.6 ** jc4340.n / 0.6
        mat = Material.STEEL_4340.yielding(jc4340.a, secant)
    mesh = QuadMesh.solidCylinder(R, L, nr, nz)
    s = cls(mesh, mat, Formulation.AXISYMMETRIC, integration, Kinematics.FINITE_STRAIN, 1.0, 0.5)
    for n in QuadMesh.axisNodes(nr, nz):
        s.fixRadial(n)
    wall = RigidWall.atZ(0.0, friction)
    s.setRigidWall(wall)
    s.setUniformVelocity(0.0, -181.0)
    return s, mesh, {"wall": wall, "length": L}


def perforation_materials():
    """Slug: 4340 elastic constants (205 GPa, 0.29), rho 7850, J2 800 MPa with 1 GPa linear
    hardening. Blocks: OFHC copper (117 GPa, 0.34, 8960) with the copper Johnson-Cook law."""
    slug = Material.STEEL_4340.yielding(800.0e6, 1.0e9)
    copper = Material.COPPER_OFHC.withJohnsonCook(JohnsonCook.COPPER_OFHC)
    return slug, copper


def perforation_inputs(cell=0.114 * MM, blocks=12, speed=700.0, weibull_modulus=10.0,
                       seed=20240611, slug_scale=0.6, copper_scale=0.9, correlation=2.0 * MM,
                       fracture_energy=20.0e3, depth=20.0 * MM, gap=6.0 * MM, damage=True):
    """Host-side inputs of the perforation scene: the assembled lattice mesh, the per-element
    materials, the initial velocities and the per-element damage data."""
    bodies = []
    for j in range(blocks):
        bodies.append(Outline.rectangle(0.0, j * 10.0 * MM, 20.0 * MM, (j + 1) * 10.0 * MM))
    midz = 0.5 * blocks * 10.0 * MM
    slug = Outline.rectangle(-10.0 * MM - gap, midz - 10.0 * MM, -gap, midz + 10.0 * MM)
    bodies.append(slug)
    mesh = Outline.assemble(cell, *bodies)
    rc, zc = mesh.centroidRadii(), mesh.centroidZs()
    isSlug = rc < 0.0
    steel, copper = perforation_materials()
    mats = Materials.of(*[steel if b else copper for b in isSlug])
    vr = np.where(mesh.r < 0.0, speed, 0.0)
    eps = gf = None
    if damage:
        eps = np.empty(mesh.elementCount)
        V0 = correlation ** 2 * depth
        for flag, scale in ((True, slug_scale), (False, copper_scale)):
            field = DefectField(Weibull(scale, weibull_modulus), V0, correlation,
                                seed + (1 if flag else 0))
            sel = isSlug == flag
            eps[sel] = field.failureStrainForVolume(rc[sel], zc[sel], V0)
        gf = np.full(mesh.elementCount, fracture_energy)
    return {"mesh": mesh, "materials": mats, "vr": vr, "vz": np.zeros(mesh.nodeCount),
            "failure_strain": eps, "fracture_energy": gf, "slug": isSlug, "depth": depth}


def perforation_build(cls, inputs, contact_friction=0.2, floor_friction=0.2, gravity=-9.81,
                      erosion=1.0, cfl=0.5):
    """The solver calls that set the perforation scene up (Smash.java:108-132)."""
    mesh = inputs["mesh"]
    s = cls(mesh, inputs["materials"], Formulation.PLANE_STRAIN, Integration.REDUCED,
            Kinematics.FINITE_STRAIN, inputs["depth"], cfl)
    if gravity:
        s.setGravity(0.0, gravity)
    wall = RigidWall.atZ(0.0, floor_friction)
    s.setRigidWall(wall)
    c = Contact(mesh).withFriction(contact_friction)
    s.setContact(c)
    s.setVelocities(inputs["vr"], inputs["vz"])
    if inputs["failure_strain"] is not None:
        s.setDamage(inputs["fracture_energy"], inputs["failure_strain"])
        if erosion:
            s.setErosion(erosion)
    return s, mesh, {"wall": wall, "contact": c, "slug": inputs["slug"]}


def perforation(cls, cell=0.114 * MM, blocks=12, speed=700.0, contact_friction=0.2,
                floor_friction=0.2, gravity=-9.81, fracture_energy=20.0e3, weibull_modulus=10.0,
                seed=20240611, slug_scale=0.6, copper_scale=0.9, correlation=2.0 * MM,
                erosion=1.0, depth=20.0 * MM, cfl=0.5, damage=True, gap=6.0 * MM):
    """A 10 x 20 mm steel slug at 700 m/s into a column of copper blocks 20 x 10 mm resting on
    a rigid floor (the Smash.main template, Smash.java:86-132). Failure strains come from a
    Weibull defect field of modulus 10 with a fixed seed, sampled at element centroids so the
    field does not depend on the mesh."""
    inputs = perforation_inputs(cell=cell, blocks=blocks, speed=speed,
                                weibull_modulus=weibull_modulus, seed=seed, slug_scale=slug_scale,
                                copper_scale=copper_scale, correlation=correlation,
                                fracture_energy=fracture_energy, depth=depth, gap=gap,
                                damage=damage)
    return perforation_build(cls, inputs, contact_friction=contact_friction,
                             floor_friction=floor_friction, gravity=gravity, erosion=erosion,
                             cfl=cfl)


def two_blocks(cls, side=10, speed=120.0, damage=True, floor=True, contact=True, cell=MM):
    """Bench.build, Bench.java:142-169."""
    half = side * cell / 2.0
    mesh = Outline.assemble(cell, Outline.rectangle(0.0, 0.0, side * cell, half),
                            Outline.rectangle(0.0, half, side * cell, side * cell))
    copper = Material.COPPER_OFHC.withJohnsonCook(JohnsonCook.COPPER_OFHC)
    s = cls(mesh, copper, Formulation.PLANE_STRAIN, Integration.REDUCED, Kinematics.FINITE_STRAIN,
            20.0 * MM, 0.5)
    if damage:
        s.setDamage(np.full(mesh.elementCount, 100.0e3), np.full(mesh.elementCount, 0.8))
        s.setErosion(1.0)
    if floor:
        s.setRigidWall(RigidWall.atZ(0.0, 0.3))
    if contact:
        s.setContact(Contact(mesh).withFriction(0.3))
    vz = np.where(mesh.z > half, -speed, 0.0)
    s.setVelocities(np.zeros(mesh.nodeCount), vz)
    return s, mesh, {}


TUBE_GF = 60.0e3


def tube_material(law=None) -> Material:
    law = law if law is not None else JohnsonCook.COPPER_OFHC.quasiStatic()
    return Material.COPPER_OFHC.withJohnsonCook(law)


def tube(cls, inner=19.6e-3, outer=20.4e-3, height=4.0e-3, nr=4, nz=20, pressure=60.0e6,
         ramp=20.0e-6, integration=Integration.FULL, kinematics=Kinematics.FINITE_STRAIN,
         damage=True, seed=7, material=None, gf=TUBE_GF, scale=0.35):
    """A pressurised thin wall with a smoothstep ramp and relaxation damping
    (DefectBurst.fire, DefectBurst.java:385-411); failure strains Weibull(scale, 10)."""
    mesh = QuadMesh.cylinderWall(inner, outer, height, nr, nz)
    copper = material if material is not None else tube_material()
    s = cls(mesh, copper, Formulation.AXISYMMETRIC, integration, kinematics, 1.0, 0.5)
    for n in QuadMesh.axialEndNodes(nr, nz):
        s.fixAxial(n)
    s.setPressureRamp(pressure, ramp)
    wave = copper.barWaveSpeed()
    s.setRelaxationDamping(0.05, wave / (0.5 * (inner + outer)))
    if damage:
        s.setDamage(np.full(mesh.elementCount, gf), tube_failure_strains(mesh, seed, scale))
    return s, mesh, {}


def tube_failure_strains(mesh, seed=7, scale=0.35):
    field = DefectField(Weibull(scale, 10.0), 1.0e-9, 1.0e-3, seed)
    return field.sampleOnto(mesh)


def tube_instance(inner=19.6e-3, outer=20.4e-3, height=4.0e-3, nr=4, nz=20, pressure=60.0e6,
                  ramp=20.0e-6, t_end=30.0e-6, damage=True, seed=7, material=None, gf=TUBE_GF,
                  scale=0.35):
    """The tube as a batch instance (reduced integration): what tube() builds."""
    from .batch import Instance
    mesh = QuadMesh.cylinderWall(inner, outer, height, nr, nz)
    copper = material if material is not None else tube_material()
    wave = copper.barWaveSpeed()
    return Instance(mesh=mesh, material=copper, t_end=t_end, hourglass=0.05,
                    fixed_axial=QuadMesh.axialEndNodes(nr, nz), pressure=(pressure, ramp),
                    damping=(0.05, wave / (0.5 * (inner + outer))),
                    damage=(gf, tube_failure_strains(mesh, seed, scale)) if damage else None)


# ---------------------------------------------------------------------------- the Taylor sweep

SWEEP_SEED = 20250611
SWEEP_T_END = 80.0e-6


class SplitMix64:
    """The SplitMix64 generator (Steele, Lea and Flood, "Fast splittable pseudorandom number
    generators", OOPSLA 2014): a Weyl sequence through a 64-bit finaliser."""

    MASK = (1 << 64) - 1

    def __init__(self, seed: int):
        self.state = seed & self.MASK

    def next(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & self.MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> float:
        return lo + (hi - lo) * ((self.next() >> 11) * (1.0 / (1 << 53)))

    def integer(self, lo: int, hi: int) -> int:
        """Uniform on lo .. hi inclusive."""
        return lo + int(self.uniform() * (hi - lo + 1))


def rod_material_with(jc: JohnsonCook) -> Material:
    """The rod steel with a drawn Johnson-Cook law; the kinematic modulus follows the law's
    secant at the fit strain, as for the 10 x 60 rod."""
    secant = jc.b * ROD_FIT_STRAIN ** jc.n / ROD_FIT_STRAIN
    base = Material("rod steel", 200.0e9, 0.29, 7850.0)
    return base.withKinematicHardening(ROD_KINEMATIC_FRACTION * secant).withJohnsonCook(jc)


def taylor_sweep(count: int = 4096, seed: int = SWEEP_SEED, t_end: float = SWEEP_T_END):
    """Draws the rods of the Taylor sweep: nr uniform on 6..24, nz on 30..120; Johnson-Cook A,
    B, n and C each uniform within +-20 % of the 10 x 60 rod's; friction uniform on [0, 0.2];
    impact speed uniform on [150, 250] m/s. Returns one dict per rod, in draw order."""
    g = SplitMix64(seed)
    rods = []
    for _ in range(count):
        nr = g.integer(6, 24)
        nz = g.integer(30, 120)
        a = ROD_JC.a * g.uniform(0.8, 1.2)
        b = ROD_JC.b * g.uniform(0.8, 1.2)
        n = ROD_JC.n * g.uniform(0.8, 1.2)
        c = ROD_JC.c * g.uniform(0.8, 1.2)
        mu = g.uniform(0.0, 0.2)
        speed = g.uniform(150.0, 250.0)
        rods.append({"nr": nr, "nz": nz, "a": a, "b": b, "n": n, "c": c, "mu": mu,
                     "speed": speed, "t_end": t_end})
    return rods


def _rod_jc(rod) -> JohnsonCook:
    j = ROD_JC
    return JohnsonCook(rod["a"], rod["b"], rod["n"], rod["c"], j.m, j.referenceStrainRate,
                       j.roomTemperature, j.meltTemperature, j.specificHeat, j.taylorQuinney)


def sweep_instances(rods, radius=3.8e-3, length=25.0e-3, hourglass=0.10):
    """The batch instances of drawn rods (what taylor_rod builds, one per rod)."""
    from .batch import Instance
    out = []
    for rod in rods:
        nr, nz = rod["nr"], rod["nz"]
        out.append(Instance(mesh=QuadMesh.solidCylinder(radius, length, nr, nz),
                            material=rod_material_with(_rod_jc(rod)), t_end=rod["t_end"],
                            velocity=(0.0, -rod["speed"]), wall=(0.0, rod["mu"]),
                            hourglass=hourglass, fixed_radial=QuadMesh.axisNodes(nr, nz)))
    return out


def sweep_rod(cls, rod, **kw):
    """One drawn rod as a single scene (the twin of its batch instance)."""
    return taylor_rod(cls, nr=rod["nr"], nz=rod["nz"], speed=rod["speed"], friction=rod["mu"],
                      material=rod_material_with(_rod_jc(rod)), **kw)


# ---------------------------------------------------------------------------- the adjoint batch

ADJOINT_SEED = 77


def adjoint_rods(count: int = 64, seed: int = ADJOINT_SEED, t_end: float = SWEEP_T_END):
    """The adjoint gradient batch: rods with the 10 x 60 rod's mesh, speed and run length, and
    Johnson-Cook constants and friction drawn as in the sweep (so every instance has its own
    gradient)."""
    rods = taylor_sweep(count, seed=seed, t_end=t_end)
    for r in rods:
        r.update(nr=10, nz=60, speed=200.0)
    return rods


def fraction_gradients(grads, rod):
    """Gradients in the (A, B, n, C, m, friction, kinematic fraction, fracture energy)
    convention of the rod's material rule H_kin = f B e^n / e (e the fit strain): chain rule
    from the adjoint's (A, B, n, C, m, H_kin, friction, fracture energy)."""
    g = np.asarray(grads, dtype=np.float64)
    b, n = rod["b"], rod["n"]
    e = ROD_FIT_STRAIN
    f = ROD_KINEMATIC_FRACTION
    secant = b * e ** n / e
    dH = g[..., 5]
    out = np.empty_like(g)
    out[..., 0] = g[..., 0]
    out[..., 1] = g[..., 1] + dH * f * e ** n / e
    out[..., 2] = g[..., 2] + dH * f * secant * math.log(e)
    out[..., 3] = g[..., 3]
    out[..., 4] = g[..., 4]
    out[..., 5] = g[..., 6]
    out[..., 6] = dH * secant
    out[..., 7:] = g[..., 7:]
    return out


# ---------------------------------------------------------------------------- burst (BurstCase)

BIAXIAL = 2.0 / math.sqrt(3.0)                      # validate/Burst.java
BIAXIAL_SOFTENING = math.sqrt(3.0)
BURST_SAMPLE_STEPS = 250                            # BurstCase.java:131-132
BURST_PEAK_MARGIN = 0.005
BURST_RAMP_PERIODS = 20.0
BURST_MAX_PERIODS = 300.0
BURST_DAMPING = 0.5
BURST_OVERSHOOT = 1.06
BURST_THROUGH_WALL = 8
BURST_ALONG_AXIS = 2
BURST_CFL = 0.5


def _instability_strain(law, softening):
    """Burst.instabilityStrain (Burst.java:100-113): dsigma/deps = softening sigma, bisected."""
    def residual(eps):
        slope = math.inf if eps <= 0.0 else law.b * law.n * math.pow(eps, law.n - 1.0)
        term = law.a if eps <= 0.0 else law.a + law.b * math.pow(eps, law.n)
        return slope - softening * term
    hi = 1.0
    lo = hi
    while residual(lo) <= 0.0:
        lo *= 0.5
        if lo < 1e-15:
            return 0.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if residual(mid) > 0.0:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def burst_pressure(law, thickness, mean_radius):
    """Burst.burstPressure (Burst.java:168-182): the thin-wall instability pressure."""
    hoop = _instability_strain(law, BIAXIAL_SOFTENING) / BIAXIAL
    eq = BIAXIAL * hoop
    term = law.a if eq <= 0.0 else law.a + law.b * math.pow(eq, law.n)
    return BIAXIAL * term * (thickness / mean_radius) * math.exp(-2.0 * hoop)


def burst_material() -> Material:
    """BurstCase.COPPER: OFHC copper on its quasi-static flow curve."""
    return Material.COPPER_OFHC.withJohnsonCook(JohnsonCook.COPPER_OFHC.quasiStatic())


def burst_instance(mean_radius=25.0e-3, slenderness=25.0, through_wall=BURST_THROUGH_WALL,
                   overshoot=BURST_OVERSHOOT, material=None):
    """BurstCase.run's tube (BurstCase.java:400-444) as a batch instance: a two-element slice
    of the wall, every node held axially, a smoothstep ramp to overshoot x the closed-form
    burst pressure over 20 ring periods, relaxation damping at the ring frequency, run to 300
    periods (the deadline)."""
    from .batch import Instance
    material = material if material is not None else burst_material()
    law = material.johnsonCook
    thickness = 2.0 * mean_radius / slenderness
    inner, outer = mean_radius - 0.5 * thickness, mean_radius + 0.5 * thickness
    h = thickness / through_wall
    mesh = QuadMesh.cylinderWall(inner, outer, h * BURST_ALONG_AXIS, through_wall,
                                 BURST_ALONG_AXIS)
    ceiling = overshoot * burst_pressure(law, thickness, mean_radius)
    omega = material.barWaveSpeed() / mean_radius
    period = 2.0 * math.pi / omega
    return Instance(mesh=mesh, material=material, t_end=BURST_MAX_PERIODS * period,
                    fixed_axial=np.arange(mesh.nodeCount), pressure=(ceiling,
                                                                    BURST_RAMP_PERIODS * period),
                    damping=(BURST_DAMPING, omega))
