"""CPU restatement of the steady-state criterion the GPU detector evaluates (a test oracle).

Windows of W recorded steps per sensor over (energy count, flux x, flux y), flux in fixed point
(2^20 units per m/s), each window split into B batches of W/B steps; a window's mean is the mean
of its batch means and its standard error their spread over sqrt(B) (sums about the previous
window's mean); window c agrees with the anchor window j when |m_c - m_j| <= z sqrt(se_c^2 +
se_j^2) for all three, and a window that disagrees becomes the anchor (window 0 is the first);
a sensor's onset is j*W for the first anchor j followed by M agreeing windows; with a trend
tolerance zd > 0 those M + 1 windows must also show no least-squares slope of any quantity's
window means beyond zd of its standard error (else the latest window becomes the anchor); the
model's onset is the largest over the sensors, -1 when any sensor has none."""
import numpy as np


def fixed_point(flux: np.ndarray) -> np.ndarray:
    return np.rint(flux * 1048576.0)


def sensor_onsets(energy: np.ndarray, flux: np.ndarray, window: int, batches: int, z: float, patience: int,
                  drift_z: float = 0.0) -> np.ndarray:
    S, K = energy.shape
    nw = K // window
    L = window // batches
    fx = fixed_point(flux[..., 0])
    fy = fixed_point(flux[..., 1])
    out = np.full(S, -1, dtype=np.int64)
    for s in range(S):
        series = [energy[s].astype(np.float64), fx[s], fy[s]]
        prev_mean = np.zeros(3)
        anchor_mean = np.zeros(3)
        anchor_se = np.zeros(3)
        anchor_w = 0
        streak = 0
        n_w = s_i = s_ii = 0.0
        s_d, s_id, v0, v1, v2 = ([0.0] * 3 for _ in range(5))
        for w in range(nw):
            mean = np.zeros(3)
            se = np.zeros(3)
            for q in range(3):
                x = series[q][w * window:(w + 1) * window] - prev_mean[q]
                bm = x.reshape(batches, L).sum(axis=1) / L
                d = bm.sum() / batches
                var = max(0.0, (np.sum(bm * bm) - batches * d * d) / (batches - 1))
                mean[q] = prev_mean[q] + d
                se[q] = np.sqrt(var / batches)
            agree = w > 0 and bool(np.all(np.abs(mean - anchor_mean) <= z * np.sqrt(se * se + anchor_se * anchor_se)))
            reset = not agree
            if agree:
                streak += 1
                i = float(streak)
                n_w += 1.0
                s_i += i
                s_ii += i * i
                for q in range(3):
                    d = mean[q] - anchor_mean[q]
                    v = se[q] * se[q]
                    s_d[q] += d
                    s_id[q] += i * d
                    v0[q] += v
                    v1[q] += i * v
                    v2[q] += i * i * v
                if streak >= patience:
                    flat = True
                    if drift_z > 0.0:
                        ib = s_i / n_w
                        sxx = s_ii - n_w * ib * ib
                        for q in range(3):
                            slope = (s_id[q] - ib * s_d[q]) / sxx
                            var = max(0.0, v2[q] - 2.0 * ib * v1[q] + ib * ib * v0[q]) / (sxx * sxx)
                            flat = flat and abs(slope) <= drift_z * np.sqrt(var)
                    if flat:
                        out[s] = anchor_w * window
                        break
                    reset = True
            if reset:
                anchor_mean, anchor_se, anchor_w, streak = mean, se, w, 0
                n_w, s_i, s_ii = 1.0, 0.0, 0.0
                s_d, s_id, v1, v2 = [0.0] * 3, [0.0] * 3, [0.0] * 3, [0.0] * 3
                v0 = [se[q] * se[q] for q in range(3)]
            prev_mean = mean
    return out


def model_onset(per_sensor: np.ndarray) -> int:
    return -1 if np.any(per_sensor < 0) else int(per_sensor.max(initial=-1))
