package org.neofiz.gpu;

/**
 * A CUDA error, a missing device, or a fault the device flagged in its status word (a
 * non-finite nodal value; a bounded wait of the contact pass that gave up, after which the
 * solver refuses to step). The reference has no counterpart: it has no device.
 */
public final class DeviceException extends RuntimeException {
    private final boolean timedOut;

    DeviceException(String message, boolean timedOut) {
        super(message);
        this.timedOut = timedOut;
    }

    /** True when a bounded device-side wait gave up (NF_ETIMEOUT). */
    public boolean timedOut() {
        return timedOut;
    }
}
