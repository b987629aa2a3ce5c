package org.neofiz.gpu;

import java.lang.foreign.Arena;
import java.lang.foreign.MemorySegment;
import java.util.List;

import org.neofiz.core.Formulation;
import org.neofiz.core.Material;
import org.neofiz.mesh.QuadMesh;
import org.neofiz.solver.Kinematics;

import static java.lang.foreign.ValueLayout.ADDRESS;
import static java.lang.foreign.ValueLayout.JAVA_BYTE;
import static java.lang.foreign.ValueLayout.JAVA_DOUBLE;
import static java.lang.foreign.ValueLayout.JAVA_INT;
import static org.neofiz.gpu.NeofizNative.*;

/**
 * A sweep of independent scenes on one GPU: what the reference runs as one ExplicitSolver per
 * host thread (Sweep.over, app/Sweep.java:82-105, over TaylorImpactCase.run :214-258). Each
 * case is the set-up sequence
 * <pre>
 *   new ExplicitSolver(mesh, material, formulation, REDUCED, kinematics, thickness, cfl)
 *   setHourglassCoefficient(q); fixRadial / fixAxial(nodes);
 *   setRigidWall(RigidWall.atZ(plane, friction)); setUniformVelocity(vr, vz);
 *   setPressureRamp(p, ramp); setRelaxationDamping(fraction, omega); setDamage(gf, eps)
 * </pre>
 * run while time &lt; tEnd, and every case computes exactly what that solver computes (FP64).
 */
public final class GpuBatch implements AutoCloseable {
    /** Arithmetic of the batched step (NF_PRECISION_*). */
    public enum Precision { FP64, MIXED, COMPENSATED }

    /** One scene of the sweep. Arrays may be empty; wallPlane NaN means no wall. */
    public record Case(QuadMesh mesh, Material material, double velocityR, double velocityZ,
                       double wallPlane, double wallFriction, double hourglass, double tEnd,
                       int[] fixedRadial, int[] fixedAxial, double pressure, double pressureRamp,
                       double dampingFraction, double dampingOmega, double[] fractureEnergy,
                       double[] failureStrain) {
        /** A Taylor rod on a Coulomb anvil (TaylorImpactCase.run's set-up). */
        public static Case taylor(QuadMesh mesh, Material material, double speed,
                                  double friction, double hourglass, double tEnd, int[] axis) {
            return new Case(mesh, material, 0.0, -speed, 0.0, friction, hourglass, tEnd, axis,
                            new int[0], 0.0, 0.0, 0.0, 0.0, null, null);
        }
    }

    private MemorySegment handle;
    private final int count;

    public GpuBatch(List<Case> cases, Formulation formulation, Kinematics kinematics,
                    double thickness, double cflSafety, Precision precision) {
        this.count = cases.size();
        int nodes = 0, elements = 0, edges = 0;
        boolean damage = cases.get(0).failureStrain() != null;
        for (Case c : cases) {
            nodes += c.mesh().nodeCount;
            elements += c.mesh().elementCount;
            edges += c.mesh().pressureEdges.length / 2;
            if ((c.failureStrain() != null) != damage)
                throw new IllegalArgumentException("damage is set on every case or on none");
        }
        try (Arena a = Arena.ofConfined()) {
            MemorySegment nodeOff = a.allocate(JAVA_INT, count + 1);
            MemorySegment elemOff = a.allocate(JAVA_INT, count + 1);
            MemorySegment presOff = a.allocate(JAVA_INT, count + 1);
            MemorySegment r = a.allocate(JAVA_DOUBLE, Math.max(1, nodes));
            MemorySegment z = a.allocate(JAVA_DOUBLE, Math.max(1, nodes));
            MemorySegment fixed = a.allocate(Math.max(1, nodes));
            MemorySegment conn = a.allocate(JAVA_INT, Math.max(1, 4L * elements));
            MemorySegment pedges = a.allocate(JAVA_INT, Math.max(1, 2L * edges));
            MemorySegment eps = damage ? a.allocate(JAVA_DOUBLE, Math.max(1, elements)) : MemorySegment.NULL;
            MemorySegment gf = damage ? a.allocate(JAVA_DOUBLE, Math.max(1, elements)) : MemorySegment.NULL;
            MemorySegment inst = a.allocate(BATCH_INSTANCE, count);
            int n0 = 0, e0 = 0, k0 = 0;
            for (int k = 0; k < count; k++) {
                Case c = cases.get(k);
                QuadMesh m = c.mesh();
                nodeOff.setAtIndex(JAVA_INT, k, n0);
                elemOff.setAtIndex(JAVA_INT, k, e0);
                presOff.setAtIndex(JAVA_INT, k, k0);
                for (int i = 0; i < m.nodeCount; i++) {
                    r.setAtIndex(JAVA_DOUBLE, n0 + i, m.r[i]);
                    z.setAtIndex(JAVA_DOUBLE, n0 + i, m.z[i]);
                }
                for (int i : c.fixedRadial())
                    fixed.set(JAVA_BYTE, n0 + i, (byte) (fixed.get(JAVA_BYTE, n0 + i) | 1));
                for (int i : c.fixedAxial())
                    fixed.set(JAVA_BYTE, n0 + i, (byte) (fixed.get(JAVA_BYTE, n0 + i) | 2));
                for (int i = 0; i < 4 * m.elementCount; i++)
                    conn.setAtIndex(JAVA_INT, 4L * e0 + i, m.conn[i]);
                for (int i = 0; i < m.pressureEdges.length; i++)
                    pedges.setAtIndex(JAVA_INT, 2L * k0 + i, m.pressureEdges[i]);
                if (damage) {
                    for (int e = 0; e < m.elementCount; e++) {
                        eps.setAtIndex(JAVA_DOUBLE, e0 + e, c.failureStrain()[e]);
                        gf.setAtIndex(JAVA_DOUBLE, e0 + e, c.fractureEnergy()[e]);
                    }
                }
                MemorySegment s = inst.asSlice(k * BATCH_INSTANCE.byteSize(), BATCH_INSTANCE.byteSize());
                GpuExplicitSolver.fillMaterial(s.asSlice(at(BATCH_INSTANCE, "material"),
                                                         MATERIAL.byteSize()), c.material());
                setD(s, BATCH_INSTANCE, "velocity_r", c.velocityR());
                setD(s, BATCH_INSTANCE, "velocity_z", c.velocityZ());
                setD(s, BATCH_INSTANCE, "wall_plane", c.wallPlane());
                setD(s, BATCH_INSTANCE, "wall_friction", c.wallFriction());
                setD(s, BATCH_INSTANCE, "hourglass", c.hourglass());
                setD(s, BATCH_INSTANCE, "t_end", c.tEnd());
                setD(s, BATCH_INSTANCE, "pressure", c.pressure());
                setD(s, BATCH_INSTANCE, "pressure_ramp", c.pressureRamp());
                setD(s, BATCH_INSTANCE, "damping_fraction", c.dampingFraction());
                setD(s, BATCH_INSTANCE, "damping_omega", c.dampingOmega());
                n0 += m.nodeCount;
                e0 += m.elementCount;
                k0 += m.pressureEdges.length / 2;
            }
            nodeOff.setAtIndex(JAVA_INT, count, n0);
            elemOff.setAtIndex(JAVA_INT, count, e0);
            presOff.setAtIndex(JAVA_INT, count, k0);
            MemorySegment bm = a.allocate(BATCH_MESH);
            setI(bm, BATCH_MESH, "instance_count", count);
            setA(bm, BATCH_MESH, "node_offset", nodeOff);
            setA(bm, BATCH_MESH, "element_offset", elemOff);
            setA(bm, BATCH_MESH, "r", r);
            setA(bm, BATCH_MESH, "z", z);
            setA(bm, BATCH_MESH, "conn", conn);
            setA(bm, BATCH_MESH, "fixed", fixed);
            setA(bm, BATCH_MESH, "pressure_offset", edges > 0 ? presOff : MemorySegment.NULL);
            setA(bm, BATCH_MESH, "pressure_edges", edges > 0 ? pedges : MemorySegment.NULL);
            setA(bm, BATCH_MESH, "failure_strain", eps);
            setA(bm, BATCH_MESH, "fracture_energy", gf);
            MemorySegment out = a.allocate(ADDRESS);
            int st = (int) BATCH_CREATE.invokeExact(bm, inst, formulation.ordinal(),
                    kinematics == Kinematics.FINITE_STRAIN ? 1 : 0, thickness, cflSafety,
                    precision.ordinal(), out);
            checkBatch(st, MemorySegment.NULL);
            this.handle = out.get(ADDRESS, 0);
        } catch (Throwable t) {
            throw rethrow(t);
        }
    }

    interface Call {
        int run() throws Throwable;
    }

    void call(Call c) {
        if (handle == null) throw new IllegalStateException("the batch has been closed");
        int st;
        try {
            st = c.run();
        } catch (Throwable t) {
            throw rethrow(t);
        }
        checkBatch(st, handle);
    }

    MemorySegment handle() {
        return handle;
    }

    public int size() {
        return count;
    }

    /** The autotuner: times every valid launch shape on trialSteps steps (the trajectory is
     * untouched) and keeps the fastest. */
    public void tune(int trialSteps) {
        try (Arena a = Arena.ofConfined()) {
            MemorySegment cfg = a.allocate(BATCH_CONFIG);
            call(() -> (int) BATCH_TUNE.invokeExact(handle, trialSteps, cfg));
        }
    }

    /** Runs every case to its tEnd (or maxSteps more steps); returns the device milliseconds. */
    public double run(long maxSteps) {
        call(() -> (int) BATCH_RUN.invokeExact(handle, maxSteps));
        try (Arena a = Arena.ofConfined()) {
            MemorySegment ms = a.allocate(JAVA_DOUBLE);
            call(() -> (int) BATCH_ELAPSED.invokeExact(handle, ms));
            return ms.get(JAVA_DOUBLE, 0);
        }
    }

    /** Per case {length, mushroomDiameter} (TaylorImpactCase.java:272-288). */
    public double[][] measure() {
        try (Arena a = Arena.ofConfined()) {
            MemorySegment m = a.allocate(MEASURE, count);
            call(() -> (int) BATCH_MEASURE.invokeExact(handle, m));
            double[][] out = new double[count][2];
            for (int k = 0; k < count; k++) {
                MemorySegment s = m.asSlice(k * MEASURE.byteSize(), MEASURE.byteSize());
                out[k][0] = getD(s, MEASURE, "length");
                out[k][1] = getD(s, MEASURE, "mushroom_diameter");
            }
            return out;
        }
    }

    @Override
    public void close() {
        if (handle == null) return;
        MemorySegment h = handle;
        handle = null;
        try {
            int st = (int) BATCH_DESTROY.invokeExact(h);
            if (st != NF_OK) throw failure(st, "nf_batch_destroy failed");
        } catch (Throwable t) {
            throw rethrow(t);
        }
    }
}
