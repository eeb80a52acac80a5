"""CPU checks of the numpy reference of the warm-start perceptron: its backward pass
equals central finite differences of its loss, and the bf16 rounding helper rounds
to nearest even."""
import numpy as np

import mlp_reference as R


def _params(rng):
    W = [rng.normal(0, np.sqrt(2.0 / i), (o, i)) for o, i in ((R.HID, R.IN), (R.HID, R.HID), (R.OUTP, R.HID))]
    W[2][R.OUT:] = 0.0
    b = [rng.normal(0, 0.1, o) for o in (R.HID, R.HID, R.OUTP)]
    b[2][R.OUT:] = 0.0
    return W, b


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.1415926], dtype=np.float32)
    y = R.bf16(x)
    assert y[0] == 1.0
    assert y[1] == 1.0                  # tie -> even
    assert y[2] == 1.0 + 2 ** -6        # tie -> even (up)
    assert y[3] == -2.5
    assert abs(y[4] - 3.140625) < 1e-7


def test_exact_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    W, b = _params(rng)
    X = rng.normal(size=(16, R.IN))
    T = rng.normal(size=(16, R.OUTP))
    T[:, R.OUT:] = 0.0
    L, dW, db = R.exact_gradients(X, T, W, b)
    for li in range(3):
        for (o, i) in [(0, 0), (3, 5), (7, 11)]:
            if li == 2 and o >= R.OUT:
                continue
            h = 1e-6
            Wp = [w.copy() for w in W]
            Wp[li][o, i] += h
            Wm = [w.copy() for w in W]
            Wm[li][o, i] -= h
            fd = (R.exact_gradients(X, T, Wp, b)[0] - R.exact_gradients(X, T, Wm, b)[0]) / (2 * h)
            assert abs(fd - dW[li][o, i]) <= 1e-6 * max(1.0, abs(fd)), (li, o, i)
        bp = [x.copy() for x in b]
        bp[li][2] += 1e-6
        bm = [x.copy() for x in b]
        bm[li][2] -= 1e-6
        fd = (R.exact_gradients(X, T, W, bp)[0] - R.exact_gradients(X, T, W, bm)[0]) / 2e-6
        assert abs(fd - db[li][2]) <= 1e-6 * max(1.0, abs(fd))


def test_rounded_backward_close_to_exact():
    """The bf16-rounded reference gradient stays within bf16 precision of the exact one."""
    rng = np.random.default_rng(4)
    W, b = _params(rng)
    X = R.bf16(rng.normal(size=(256, R.IN)).astype(np.float32))
    T = rng.normal(size=(256, R.OUTP))
    T[:, R.OUT:] = 0.0
    Wr = [R.bf16(w.astype(np.float32)).astype(np.float64) for w in W]
    Y, acts = R.forward(X, W, b)
    _, dY = R.loss_and_dy(Y, T)
    dW, _ = R.backward(acts, dY, W)
    _, dWe, _ = R.exact_gradients(X.astype(np.float64), T, Wr, b)
    for li in range(3):
        err = np.max(np.abs(dW[li] - dWe[li])) / np.max(np.abs(dWe[li]))
        assert err < 0.03, (li, err)
