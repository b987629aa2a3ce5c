package org.neofiz.gpu;

import org.neofiz.mesh.QuadMesh;

/**
 * The reference's {@code Contact} (Contact.java:136-404) for a {@link GpuExplicitSolver}: the
 * same builder and statistics, with the reference's validation messages. The contact state
 * (surface, search grid, pairs) lives on the device with the solver it was handed to.
 */
public final class GpuContact {
    /** Contact.DEFAULT_SCALE, Contact.java:143. */
    public static final double DEFAULT_SCALE = 0.1;
    /** Contact.DEFAULT_DAMPING, Contact.java:207. */
    public static final double DEFAULT_DAMPING = 0.0;

    private final QuadMesh mesh;
    private final double friction;
    private final double damping;
    private final double scale;
    private GpuExplicitSolver solver;

    public GpuContact(QuadMesh mesh) {
        this(mesh, 0.0, DEFAULT_DAMPING, DEFAULT_SCALE);
    }

    private GpuContact(QuadMesh mesh, double friction, double damping, double scale) {
        this.mesh = mesh;
        this.friction = friction;
        this.damping = damping;
        this.scale = scale;
    }

    /** withFriction, Contact.java:335-344. */
    public GpuContact withFriction(double mu) {
        if (mu < 0.0) throw new IllegalArgumentException("friction must not be negative");
        return new GpuContact(mesh, mu, damping, scale);
    }

    /** withDamping, Contact.java:346-353. */
    public GpuContact withDamping(double zeta) {
        if (zeta < 0.0 || zeta > 1.0)
            throw new IllegalArgumentException(
                    "contact damping is a fraction of critical, so it lies in [0, 1]; was " + zeta);
        return new GpuContact(mesh, friction, zeta, scale);
    }

    /** withStiffnessScale, Contact.java:355-364. */
    public GpuContact withStiffnessScale(double s) {
        if (!(s > 0.0) || s >= 2.0)
            throw new IllegalArgumentException("the stiffness scale must lie in (0, 2); a pair is "
                    + "found from both sides, so the effective stiffness is twice this and above 2 "
                    + "the contact frequency exceeds what central difference can integrate, was " + s);
        return new GpuContact(mesh, friction, damping, s);
    }

    void bind(GpuExplicitSolver s) {
        this.solver = s;
    }

    public double friction() {
        return friction;
    }

    double damping() {
        return damping;
    }

    double stiffnessScale() {
        return scale;
    }

    public int pairCount() {
        return solver == null ? 0 : (int) solver.contactStat("pair_count");
    }

    public double energy() {
        return solver == null ? 0.0 : solver.contactStat("energy");
    }

    public double dissipation() {
        return solver == null ? 0.0 : solver.contactStat("dissipation");
    }

    public double maxPenetration() {
        return solver == null ? 0.0 : solver.contactStat("max_penetration");
    }

    public int escapedNodes() {
        return solver == null ? 0 : (int) solver.contactStat("escaped_nodes");
    }

    public int segmentCount() {
        return solver == null ? 0 : (int) solver.contactStat("segment_count");
    }
}
