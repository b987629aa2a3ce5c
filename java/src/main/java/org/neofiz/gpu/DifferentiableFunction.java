package org.neofiz.gpu;

import java.util.function.Function;

/**
 * A function with a hand-written reverse, in the style of an autograd Function: {@code
 * forward(x)} computes y and keeps what the reverse needs; {@code backward(dy)} then returns
 * the vector-Jacobian product dy^T (dy/dx), shaped like x. As a {@link Function} it is its
 * forward half.
 *
 * @param <X> the input (and gradient) type
 * @param <Y> the output (and seed) type
 */
public interface DifferentiableFunction<X, Y> extends Function<X, Y> {
    Y forward(X input);

    /** The gradient, with respect to the last forward call's input, of seed . output. */
    X backward(Y seed);

    @Override
    default Y apply(X input) {
        return forward(input);
    }
}
