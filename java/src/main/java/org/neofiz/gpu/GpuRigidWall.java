package org.neofiz.gpu;

/**
 * The reference's {@code RigidWall} (RigidWall.java:110-315) for a {@link GpuExplicitSolver}:
 * the same factories and statistics. The wall's state lives on the device with the solver it
 * was handed to; until then the statistics are zero.
 */
public final class GpuRigidWall {
    private final double plane;
    private final double friction;
    private GpuExplicitSolver solver;

    private GpuRigidWall(double plane, double friction) {
        if (friction < 0.0 || Double.isNaN(friction))
            throw new IllegalArgumentException("friction coefficient must be >= 0");
        this.plane = plane;
        this.friction = friction;
    }

    /** RigidWall.atZ(z), :121-123: frictionless. */
    public static GpuRigidWall atZ(double z) {
        return new GpuRigidWall(z, 0.0);
    }

    /** RigidWall.atZ(z, friction), :134-136; friction = +infinity is the welded limit. */
    public static GpuRigidWall atZ(double z, double friction) {
        return new GpuRigidWall(z, friction);
    }

    void bind(GpuExplicitSolver s) {
        this.solver = s;
    }

    public double plane() {
        return plane;
    }

    public double friction() {
        return friction;
    }

    public boolean hasFriction() {
        return friction > 0.0;
    }

    public double impulse() {
        return solver == null ? 0.0 : solver.wallStat("impulse");
    }

    public double energyLoss() {
        return solver == null ? 0.0 : solver.wallStat("energy_loss");
    }

    public double frictionDissipation() {
        return solver == null ? 0.0 : solver.wallStat("friction_dissipation");
    }

    public int contactCount() {
        return solver == null ? 0 : (int) solver.wallStat("contact_count");
    }

    public int stuckCount() {
        return solver == null ? 0 : (int) solver.wallStat("stuck_count");
    }
}
