package org.neofiz.gpu;

import java.lang.foreign.Arena;
import java.lang.foreign.MemorySegment;
import java.util.List;

import org.neofiz.core.Formulation;
import org.neofiz.core.JohnsonCook;
import org.neofiz.core.Material;
import org.neofiz.core.Materials;
import org.neofiz.mesh.QuadMesh;
import org.neofiz.solver.Integration;
import org.neofiz.solver.Kinematics;

import static java.lang.foreign.ValueLayout.ADDRESS;
import static java.lang.foreign.ValueLayout.JAVA_BYTE;
import static java.lang.foreign.ValueLayout.JAVA_DOUBLE;
import static java.lang.foreign.ValueLayout.JAVA_INT;
import static java.lang.foreign.ValueLayout.JAVA_LONG;
import static org.neofiz.gpu.NeofizNative.*;

/**
 * The reference's {@code org.neofiz.solver.ExplicitSolver} (ExplicitSolver.java:237-1936) on
 * the GPU: the same constructors, setters, run methods, getters and audits, each a call into
 * libneofiz_gpu.so. The timestep runs on the device bit for bit as the Java one does.
 *
 * <p>What a caller sees differently, all because the state lives on the device:
 * <ul>
 *   <li>getters return copies, not live arrays (a caller that wrote into a live array uses
 *       {@link #setVelocity} or {@link #writeField});</li>
 *   <li>{@code setThreads} is accepted and ignored: the device is the parallelism;</li>
 *   <li>{@link GpuRigidWall} and {@link GpuContact} replace RigidWall and Contact: the same
 *       factories and statistics, read from the solver they were handed to;</li>
 *   <li>run methods only enqueue; reads wait for them. {@link #close()} frees the device
 *       memory (the reference's {@code shutdown}).</li>
 * </ul>
 *
 * <p>A caller switches by constructing this class where it constructed ExplicitSolver
 * (TaylorImpactCase.run :232-258, Smash.main :108-162, Bench.build :142-169,
 * DefectBurst.fire :385-446); ExplicitSolver is final, so this is a sibling class.
 */
public final class GpuExplicitSolver implements AutoCloseable {
    private MemorySegment handle;
    private final QuadMesh mesh;
    private final Integration integration;
    private final Kinematics kinematics;
    private final Formulation formulation;
    private GpuRigidWall wall;
    private GpuContact contact;

    public GpuExplicitSolver(QuadMesh mesh, Material material, Formulation formulation,
                             Integration integration, Kinematics kinematics, double thickness,
                             double cflSafety) {
        this(mesh, Materials.uniform(material), formulation, integration, kinematics, thickness,
             cflSafety);
    }

    /** ExplicitSolver(QuadMesh, Materials, ...), ExplicitSolver.java:264-339. */
    public GpuExplicitSolver(QuadMesh mesh, Materials materials, Formulation formulation,
                             Integration integration, Kinematics kinematics, double thickness,
                             double cflSafety) {
        this.mesh = mesh;
        this.formulation = formulation;
        this.integration = integration;
        this.kinematics = kinematics;
        try (Arena a = Arena.ofConfined()) {
            MemorySegment m = a.allocate(MESH);
            setI(m, MESH, "node_count", mesh.nodeCount);
            setI(m, MESH, "element_count", mesh.elementCount);
            setI(m, MESH, "pressure_edge_count", mesh.pressureEdges.length / 2);
            setA(m, MESH, "r", a.allocateFrom(JAVA_DOUBLE, mesh.r));
            setA(m, MESH, "z", a.allocateFrom(JAVA_DOUBLE, mesh.z));
            setA(m, MESH, "conn", a.allocateFrom(JAVA_INT, mesh.conn));
            setA(m, MESH, "pressure_edges", mesh.pressureEdges.length == 0
                    ? MemorySegment.NULL : a.allocateFrom(JAVA_INT, mesh.pressureEdges));
            materials.requireCovers(mesh.elementCount);
            List<Material> distinct = materials.distinct();
            MemorySegment table = a.allocate(MATERIAL, distinct.size());
            for (int k = 0; k < distinct.size(); k++)
                fillMaterial(table.asSlice(k * MATERIAL.byteSize(), MATERIAL.byteSize()),
                             distinct.get(k));
            MemorySegment index = a.allocate(JAVA_INT, mesh.elementCount);
            for (int e = 0; e < mesh.elementCount; e++)
                index.setAtIndex(JAVA_INT, e, distinct.indexOf(materials.at(e)));
            MemorySegment out = a.allocate(ADDRESS);
            int st = (int) CREATE.invokeExact(m, table, distinct.size(), index,
                    formulation.ordinal(), integration == Integration.FULL ? 0 : 1,
                    kinematics == Kinematics.FINITE_STRAIN ? 1 : 0, thickness, cflSafety, out);
            check(st, MemorySegment.NULL);
            this.handle = out.get(ADDRESS, 0);
        } catch (Throwable t) {
            throw rethrow(t);
        }
    }

    /** Writes a Material record (Material.java:17-21, JohnsonCook.java:68-71) as nf_material. */
    static void fillMaterial(MemorySegment s, Material m) {
        setD(s, MATERIAL, "youngs_modulus", m.youngsModulus());
        setD(s, MATERIAL, "poisson_ratio", m.poissonRatio());
        setD(s, MATERIAL, "density", m.density());
        setD(s, MATERIAL, "yield_stress", m.yieldStress());
        setD(s, MATERIAL, "isotropic_hardening", m.isotropicHardening());
        setD(s, MATERIAL, "kinematic_hardening", m.kinematicHardening());
        JohnsonCook jc = m.johnsonCook();
        setI(s, MATERIAL, "has_johnson_cook", jc == null ? 0 : 1);
        if (jc != null) {
            setD(s, MATERIAL, "jc_a", jc.a());
            setD(s, MATERIAL, "jc_b", jc.b());
            setD(s, MATERIAL, "jc_n", jc.n());
            setD(s, MATERIAL, "jc_c", jc.c());
            setD(s, MATERIAL, "jc_m", jc.m());
            setD(s, MATERIAL, "jc_reference_strain_rate", jc.referenceStrainRate());
            setD(s, MATERIAL, "jc_room_temperature", jc.roomTemperature());
            setD(s, MATERIAL, "jc_melt_temperature", jc.meltTemperature());
            setD(s, MATERIAL, "jc_specific_heat", jc.specificHeat());
            setD(s, MATERIAL, "jc_taylor_quinney", jc.taylorQuinney());
        }
    }

    // ------------------------------------------------------------------ plumbing

    private interface Call {
        int run() throws Throwable;
    }

    private void call(Call c) {
        if (handle == null) throw new IllegalStateException("the solver has been shut down");
        int st;
        try {
            st = c.run();
        } catch (Throwable t) {
            throw rethrow(t);
        }
        check(st, handle);
    }

    MemorySegment handle() {
        return handle;
    }

    /** A field copied device to host (nf_read_field), as doubles. */
    public double[] readDoubles(int field) {
        try (Arena a = Arena.ofConfined()) {
            MemorySegment count = a.allocate(JAVA_LONG), bytes = a.allocate(JAVA_LONG);
            call(() -> (int) FIELD_SIZE.invokeExact(handle, field, count, bytes));
            long n = count.get(JAVA_LONG, 0);
            MemorySegment dst = a.allocate(JAVA_DOUBLE, Math.max(1, n));
            call(() -> (int) READ_FIELD.invokeExact(handle, field, dst, 8L * n));
            return n == 0 ? new double[0] : dst.asSlice(0, 8L * n).toArray(JAVA_DOUBLE);
        }
    }

    /** A byte-per-entry field (eroded, on-wall, fixed flags). */
    public byte[] readBytes(int field) {
        try (Arena a = Arena.ofConfined()) {
            MemorySegment count = a.allocate(JAVA_LONG), bytes = a.allocate(JAVA_LONG);
            call(() -> (int) FIELD_SIZE.invokeExact(handle, field, count, bytes));
            long n = count.get(JAVA_LONG, 0);
            MemorySegment dst = a.allocate(Math.max(1, n));
            call(() -> (int) READ_FIELD.invokeExact(handle, field, dst, n));
            return n == 0 ? new byte[0] : dst.asSlice(0, n).toArray(JAVA_BYTE);
        }
    }

    /** An int-per-entry field (contact masters, surface lists). */
    public int[] readInts(int field) {
        try (Arena a = Arena.ofConfined()) {
            MemorySegment count = a.allocate(JAVA_LONG), bytes = a.allocate(JAVA_LONG);
            call(() -> (int) FIELD_SIZE.invokeExact(handle, field, count, bytes));
            long n = count.get(JAVA_LONG, 0);
            MemorySegment dst = a.allocate(JAVA_INT, Math.max(1, n));
            call(() -> (int) READ_FIELD.invokeExact(handle, field, dst, 4L * n));
            return n == 0 ? new int[0] : dst.asSlice(0, 4L * n).toArray(JAVA_INT);
        }
    }

    /** Overwrites a state field host to device: the writes callers made into live arrays. */
    public void writeField(int field, double[] values) {
        try (Arena a = Arena.ofConfined()) {
            MemorySegment src = a.allocateFrom(JAVA_DOUBLE, values);
            call(() -> (int) WRITE_FIELD.invokeExact(handle, field, src, 8L * values.length));
        }
    }

    private MemorySegment struct(java.lang.foreign.StructLayout layout, java.lang.invoke.MethodHandle h,
                                 Arena a) {
        MemorySegment s = a.allocate(layout);
        call(() -> (int) h.invokeExact(handle, s));
        return s;
    }

    private double state(String name) {
        try (Arena a = Arena.ofConfined()) {
            return getD(struct(STATE, GET_STATE, a), STATE, name);
        }
    }

    private double audit(String name) {
        try (Arena a = Arena.ofConfined()) {
            return getD(struct(AUDIT, AUDITS, a), AUDIT, name);
        }
    }

    double wallStat(String name) {
        try (Arena a = Arena.ofConfined()) {
            MemorySegment s = struct(WALL_INFO, WALL_STATS, a);
            return name.endsWith("_count") ? getI(s, WALL_INFO, name) : getD(s, WALL_INFO, name);
        }
    }

    double contactStat(String name) {
        try (Arena a = Arena.ofConfined()) {
            MemorySegment s = struct(CONTACT_INFO, CONTACT_STATS, a);
            return name.endsWith("_count") || name.endsWith("_nodes")
                    ? getI(s, CONTACT_INFO, name) : getD(s, CONTACT_INFO, name);
        }
    }

    // ------------------------------------------------------------------ lifecycle (:386-403)

    /** Accepted for signature compatibility; the device is the parallelism. */
    public void setThreads(int n) {
        if (n < 1) throw new IllegalArgumentException("threads must be >= 1");
    }

    public int threads() {
        return 1;
    }

    public void shutdown() {
        close();
    }

    @Override
    public void close() {
        if (handle == null) return;
        MemorySegment h = handle;
        handle = null;
        try {
            int st = (int) DESTROY.invokeExact(h);
            if (st != NF_OK) throw failure(st, "nf_destroy failed");
        } catch (Throwable t) {
            throw rethrow(t);
        }
    }

    // ------------------------------------------------------------------ set-up (:408-808)

    public void fixRadial(int node) {
        call(() -> (int) FIX_RADIAL.invokeExact(handle, node));
    }

    public void fixAxial(int node) {
        call(() -> (int) FIX_AXIAL.invokeExact(handle, node));
    }

    public void fixAllAxial() {
        call(() -> (int) FIX_ALL_AXIAL.invokeExact(handle));
    }

    public void setPressureRamp(double pascals, double rampSeconds) {
        call(() -> (int) SET_PRESSURE_RAMP.invokeExact(handle, pascals, rampSeconds));
    }

    public void setRelaxationDamping(double fractionOfCritical, double angularFrequency) {
        call(() -> (int) SET_RELAXATION_DAMPING.invokeExact(handle, fractionOfCritical,
                                                             angularFrequency));
    }

    public void setHourglassCoefficient(double q) {
        call(() -> (int) SET_HOURGLASS.invokeExact(handle, q));
    }

    /** setRigidWall, :475-477; null removes the wall. */
    public void setRigidWall(GpuRigidWall w) {
        if (w == null) {
            call(() -> (int) CLEAR_RIGID_WALL.invokeExact(handle));
        } else {
            call(() -> (int) SET_RIGID_WALL.invokeExact(handle, w.plane(), w.friction()));
            w.bind(this);
        }
        this.wall = w;
    }

    /** setContact, :487-489; null removes contact. */
    public void setContact(GpuContact c) {
        if (c == null) {
            call(() -> (int) CLEAR_CONTACT.invokeExact(handle));
        } else {
            call(() -> (int) SET_CONTACT.invokeExact(handle, c.friction(), c.damping(),
                                                      c.stiffnessScale()));
            c.bind(this);
        }
        this.contact = c;
    }

    public GpuContact contact() {
        return contact;
    }

    public void setGravity(double accelerationR, double accelerationZ) {
        call(() -> (int) SET_GRAVITY.invokeExact(handle, accelerationR, accelerationZ));
    }

    public void setErosion(double damageThreshold) {
        call(() -> (int) SET_EROSION.invokeExact(handle, damageThreshold));
    }

    public void setMassScaling(double targetStep) {
        call(() -> (int) SET_MASS_SCALING.invokeExact(handle, targetStep));
    }

    public double massScale() {
        return state("mass_scale");
    }

    /** setDamage(double fractureEnergy, double[] failureStrain), :713-727. */
    public void setDamage(double fractureEnergy, double[] failureStrain) {
        double[] gf = new double[mesh.elementCount];
        java.util.Arrays.fill(gf, fractureEnergy);
        setDamage(gf, failureStrain);
    }

    /** setDamage(double[] fractureEnergy, double[] failureStrain), :729-791. */
    public void setDamage(double[] fractureEnergy, double[] failureStrain) {
        if (fractureEnergy.length != mesh.elementCount || failureStrain.length != mesh.elementCount)
            throw new IllegalArgumentException("one value per element is needed");
        try (Arena a = Arena.ofConfined()) {
            MemorySegment gf = a.allocateFrom(JAVA_DOUBLE, fractureEnergy);
            MemorySegment eps = a.allocateFrom(JAVA_DOUBLE, failureStrain);
            call(() -> (int) SET_DAMAGE.invokeExact(handle, gf, eps));
        }
    }

    public void setVelocity(int node, double velocityR, double velocityZ) {
        call(() -> (int) SET_VELOCITY.invokeExact(handle, node, velocityR, velocityZ));
    }

    public void setUniformVelocity(double velocityR, double velocityZ) {
        call(() -> (int) SET_UNIFORM_VELOCITY.invokeExact(handle, velocityR, velocityZ));
    }

    public Integration integration() {
        return integration;
    }

    public Kinematics kinematics() {
        return kinematics;
    }

    public Formulation formulation() {
        return formulation;
    }

    // ------------------------------------------------------------------ run (:936-1075)

    public void run(int steps) {
        call(() -> (int) STEP.invokeExact(handle, (long) steps));
    }

    public void step() {
        run(1);
    }

    public void advance() {
        call(() -> (int) ADVANCE.invokeExact(handle));
    }

    /** The loop {@code while (time() < tEnd) step();} (TaylorImpactCase.java:250-253), with
     * the test made on the device; returns the steps taken. */
    public long runUntil(double tEnd) {
        try (Arena a = Arena.ofConfined()) {
            MemorySegment taken = a.allocate(JAVA_LONG);
            call(() -> (int) RUN_UNTIL.invokeExact(handle, tEnd, Long.MAX_VALUE, taken));
            return taken.get(JAVA_LONG, 0);
        }
    }

    /** Waits for the enqueued steps; throws DeviceException if a contact-pass wait gave up. */
    public void synchronize() {
        call(() -> (int) SYNCHRONIZE.invokeExact(handle));
    }

    /** Waits, then raises the device's status word: a non-finite nodal value or a wait that
     * gave up. Callers check this on sampled frames; the reference lets NaNs propagate. */
    public void checkDevice() {
        call(() -> (int) CHECK.invokeExact(handle));
    }

    // ------------------------------------------------------------------ getters (:622-932)

    public double timestep() {
        return state("timestep");
    }

    public double time() {
        return state("time");
    }

    public long steps() {
        try (Arena a = Arena.ofConfined()) {
            return struct(STATE, GET_STATE, a).get(JAVA_LONG, at(STATE, "steps"));
        }
    }

    public double borePressure() {
        return state("bore_pressure");
    }

    public int erodedElements() {
        try (Arena a = Arena.ofConfined()) {
            return getI(struct(STATE, GET_STATE, a), STATE, "eroded_elements");
        }
    }

    public int invertedElements() {
        try (Arena a = Arena.ofConfined()) {
            return getI(struct(STATE, GET_STATE, a), STATE, "inverted_elements");
        }
    }

    public double erodedEnergy() {
        return state("eroded_energy");
    }

    public boolean isEroded(int element) {
        return readBytes(FIELD_ERODED)[element] != 0;
    }

    public double[] radialDisplacement() {
        return readDoubles(FIELD_UR);
    }

    public double[] axialDisplacement() {
        return readDoubles(FIELD_UZ);
    }

    public double[] velocityR() {
        return readDoubles(FIELD_VR);
    }

    public double[] velocityZ() {
        return readDoubles(FIELD_VZ);
    }

    public double[] forceR() {
        return readDoubles(FIELD_FR);
    }

    public double[] forceZ() {
        return readDoubles(FIELD_FZ);
    }

    public double[] plasticStrain() {
        return readDoubles(FIELD_PLASTIC_STRAIN);
    }

    /** Four components {rr, zz, theta-theta, rz} per integration point. */
    public double[] stress() {
        return readDoubles(FIELD_STRESS);
    }

    public double[] plasticWorkDensity() {
        return readDoubles(FIELD_PLASTIC_WORK);
    }

    /** centroidStress, :1886-1894: the mean of the element's points. */
    public double[] centroidStress(int element) {
        double[] s = stress();
        int ppe = integration == Integration.FULL ? 4 : 1;
        double[] out = new double[4];
        for (int g = 0; g < ppe; g++)
            for (int k = 0; k < 4; k++) out[k] += s[4 * (element * ppe + g) + k];
        for (int k = 0; k < 4; k++) out[k] /= ppe;
        return out;
    }

    /** elementPlasticStrain, :1897-1901. */
    public double elementPlasticStrain(int element) {
        double[] e = plasticStrain();
        int ppe = integration == Integration.FULL ? 4 : 1;
        double sum = 0.0;
        for (int g = 0; g < ppe; g++) sum += e[element * ppe + g];
        return sum / ppe;
    }

    // ------------------------------------------------------------------ audits (:875-886, :1610-1860)

    public double kineticEnergy() {
        return audit("kinetic_energy");
    }

    public double centredKineticEnergy() {
        return audit("centred_kinetic_energy");
    }

    public double strainEnergy() {
        return audit("strain_energy");
    }

    public double plasticDissipation() {
        return audit("plastic_dissipation");
    }

    public double hourglassEnergy() {
        return audit("hourglass_energy");
    }

    public double fractureDissipation() {
        return audit("fracture_dissipation");
    }

    public double axialMomentum() {
        return audit("axial_momentum");
    }

    public double radialMomentum() {
        return audit("radial_momentum");
    }

    public double maxPlasticStrain() {
        return audit("max_plastic_strain");
    }

    public double yieldedFraction() {
        return audit("yielded_fraction");
    }

    public double maxDamage() {
        return audit("max_damage");
    }

    public double damagedFraction() {
        return audit("damaged_fraction");
    }

    public double failedFraction() {
        return audit("failed_fraction");
    }

    public double maxTemperature() {
        return audit("max_temperature");
    }

    public int mostDamagedElement() {
        try (Arena a = Arena.ofConfined()) {
            return getI(struct(AUDIT, AUDITS, a), AUDIT, "most_damaged_element");
        }
    }

    /** TaylorImpactCase's measurements (:272-288): the body's axial extent and its widest
     * diameter 2 max(r + ur), in metres, as {length, mushroomDiameter}. */
    public double[] measure() {
        try (Arena a = Arena.ofConfined()) {
            MemorySegment s = struct(MEASURE, MEASURE_BODY, a);
            return new double[] {getD(s, MEASURE, "length"), getD(s, MEASURE, "mushroom_diameter")};
        }
    }
}
