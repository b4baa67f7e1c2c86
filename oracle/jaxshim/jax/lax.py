"""``jax.lax`` control flow as plain Python control flow (test infrastructure)."""


def while_loop(cond_fun, body_fun, init_val):
    value = init_val
    while bool(cond_fun(value)):
        value = body_fun(value)
    return value


def fori_loop(lower, upper, body_fun, init_val):
    value = init_val
    for index in range(int(lower), int(upper)):
        value = body_fun(index, value)
    return value


def cond(pred, true_fun, false_fun, *operands):
    return true_fun(*operands) if bool(pred) else false_fun(*operands)
