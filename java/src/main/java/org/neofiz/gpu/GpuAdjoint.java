package org.neofiz.gpu;

import java.lang.foreign.Arena;
import java.lang.foreign.MemorySegment;
import java.util.List;
import java.util.function.Function;

import org.neofiz.core.Formulation;
import org.neofiz.mesh.QuadMesh;
import org.neofiz.solver.Kinematics;

import static java.lang.foreign.ValueLayout.JAVA_DOUBLE;
import static java.lang.foreign.ValueLayout.JAVA_INT;
import static org.neofiz.gpu.NeofizNative.*;

/**
 * Gradients of a sweep's final measurements with respect to material and wall parameters, by
 * the library's hand-written reverse sweep of the whole timestep (nf_batch_adjoint_*; the
 * reference has no adjoint). Behind the {@link DifferentiableFunction} interface:
 * <pre>
 *   var f = new GpuAdjoint(params -&gt; casesFor(params), Formulation.AXISYMMETRIC,
 *                          Kinematics.FINITE_STRAIN, 1.0, 0.6, Objective.LENGTH_RATIO, 200, 0);
 *   double[] ratios = f.forward(params);          // one L/L0 per case
 *   double[][] grads = f.backward(ones);          // d(L/L0)/d(A, B, n, C, m, H_kin, mu, ...)
 * </pre>
 * The input is one parameter vector per case ({@link Parameter} order, NF_PARAM_COUNT
 * entries); the caller's function turns the vectors into the cases of a batch (the template
 * of the sweep). forward runs every case to its tEnd keeping a checkpoint every
 * checkpointEvery steps; backward recomputes the segments and runs the adjoint of every step in
 * reverse, with the forward pass's decisions frozen: each point's elastic/plastic branch and
 * rate and temperature clamps, each wall node's hold/stick/slip/arrive state and the element
 * that sets each CFL step. Each case's objective depends only on its own parameters, so the
 * vector-Jacobian product is the seed of each case times its gradient.
 */
public final class GpuAdjoint implements DifferentiableFunction<double[][], double[]>, AutoCloseable {
    /** NF_OBJECTIVE_*: L/L0 (TaylorImpactCase.java:272-279), 2 max(r + ur) (:281-288), the
     * largest sampled BurstCase.loadCapacity (BurstCase.java:533-553). */
    public enum Objective { LENGTH_RATIO, MUSHROOM_DIAMETER, PEAK_CAPACITY }

    /** NF_PARAM_*: Johnson-Cook A, B, n, C, m; the kinematic hardening modulus; the wall
     * friction; the fracture energy; the yield stress and isotropic modulus of a material
     * without a Johnson-Cook law. */
    public enum Parameter { A, B, N, C, M, KINEMATIC_MODULUS, FRICTION, FRACTURE_ENERGY,
                            YIELD_STRESS, ISOTROPIC_MODULUS }

    public static final int PARAMETERS = Parameter.values().length;

    private final Function<double[][], List<GpuBatch.Case>> template;
    private final Formulation formulation;
    private final Kinematics kinematics;
    private final double thickness, cfl;
    private final Objective objective;
    private final int checkpointEvery, sampleEvery;
    private GpuBatch batch;
    private double[] values;
    private double[][] gradients;

    public GpuAdjoint(Function<double[][], List<GpuBatch.Case>> template, Formulation formulation,
                      Kinematics kinematics, double thickness, double cfl, Objective objective,
                      int checkpointEvery, int sampleEvery) {
        if (objective == Objective.PEAK_CAPACITY && sampleEvery <= 0)
            throw new IllegalArgumentException("the peak capacity needs a sampling interval");
        this.template = template;
        this.formulation = formulation;
        this.kinematics = kinematics;
        this.thickness = thickness;
        this.cfl = cfl;
        this.objective = objective;
        this.checkpointEvery = checkpointEvery;
        this.sampleEvery = sampleEvery;
    }

    /** Runs the cases built from these parameters forward, with checkpoints; returns the
     * objective of every case. */
    @Override
    public double[] forward(double[][] parameters) {
        close();
        List<GpuBatch.Case> cases = template.apply(parameters);
        batch = new GpuBatch(cases, formulation, kinematics, thickness, cfl, GpuBatch.Precision.FP64);
        batch.call(() -> (int) BATCH_ADJOINT_FORWARD.invokeExact(batch.handle(), checkpointEvery,
                                                                  sampleEvery));
        gradients = null;
        if (objective == Objective.PEAK_CAPACITY) {
            reverse();                       // the sampled peak is known after the reverse only
            return values.clone();
        }
        double[][] m = batch.measure();
        values = new double[cases.size()];
        for (int k = 0; k < values.length; k++) {
            values[k] = objective == Objective.LENGTH_RATIO
                    ? m[k][0] / initialLength(cases.get(k).mesh()) : m[k][1];
        }
        return values.clone();
    }

    /** seed[k] times the gradient of case k's objective, for every case and parameter. */
    @Override
    public double[][] backward(double[] seed) {
        if (batch == null) throw new IllegalStateException("backward before forward");
        if (gradients == null) reverse();
        double[][] out = new double[gradients.length][PARAMETERS];
        for (int k = 0; k < out.length; k++)
            for (int p = 0; p < PARAMETERS; p++) out[k][p] = seed[k] * gradients[k][p];
        return out;
    }

    /** The gradient rows themselves (seed 1 for every case). */
    public double[][] jacobian() {
        double[] ones = new double[batch.size()];
        java.util.Arrays.fill(ones, 1.0);
        return backward(ones);
    }

    private void reverse() {
        int n = batch.size();
        try (Arena a = Arena.ofConfined()) {
            MemorySegment v = a.allocate(JAVA_DOUBLE, n);
            MemorySegment g = a.allocate(JAVA_DOUBLE, (long) n * PARAMETERS);
            batch.call(() -> (int) BATCH_ADJOINT_BACKWARD.invokeExact(batch.handle(),
                                                                       objective.ordinal(), v, g));
            values = v.toArray(JAVA_DOUBLE);
            double[] flat = g.toArray(JAVA_DOUBLE);
            gradients = new double[n][PARAMETERS];
            for (int k = 0; k < n; k++)
                System.arraycopy(flat, k * PARAMETERS, gradients[k], 0, PARAMETERS);
        }
    }

    /** Device milliseconds of the last forward and backward passes. */
    public double[] elapsed() {
        try (Arena a = Arena.ofConfined()) {
            MemorySegment f = a.allocate(JAVA_DOUBLE), b = a.allocate(JAVA_DOUBLE);
            batch.call(() -> (int) BATCH_ADJOINT_ELAPSED.invokeExact(batch.handle(), f, b));
            return new double[] {f.get(JAVA_DOUBLE, 0), b.get(JAVA_DOUBLE, 0)};
        }
    }

    private static double initialLength(QuadMesh m) {
        double lo = Double.POSITIVE_INFINITY, hi = Double.NEGATIVE_INFINITY;
        for (double z : m.z) {
            lo = Math.min(lo, z);
            hi = Math.max(hi, z);
        }
        return hi - lo;
    }

    @Override
    public void close() {
        if (batch != null) batch.close();
        batch = null;
    }

    /** Several objectives of one forward pass through one recompute of the segments
     * (nf_batch_adjoint_backward_many): [objective][case][parameter]. */
    public double[][][] jacobians(Objective... objectives) {
        if (batch == null) throw new IllegalStateException("jacobians before forward");
        int n = batch.size(), w = objectives.length;
        try (Arena a = Arena.ofConfined()) {
            MemorySegment obj = a.allocate(JAVA_INT, w);
            for (int i = 0; i < w; i++) obj.setAtIndex(JAVA_INT, i, objectives[i].ordinal());
            MemorySegment v = a.allocate(JAVA_DOUBLE, (long) w * n);
            MemorySegment g = a.allocate(JAVA_DOUBLE, (long) w * n * PARAMETERS);
            batch.call(() -> (int) BATCH_ADJOINT_BACKWARD_MANY.invokeExact(batch.handle(), obj, w,
                                                                            v, g));
            double[] flat = g.toArray(JAVA_DOUBLE);
            double[][][] out = new double[w][n][PARAMETERS];
            for (int i = 0; i < w; i++)
                for (int k = 0; k < n; k++)
                    System.arraycopy(flat, (i * n + k) * PARAMETERS, out[i][k], 0, PARAMETERS);
            return out;
        }
    }
}
