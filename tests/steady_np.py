"""CPU restatement of the steady-state criterion the GPU detector evaluates (a test oracle).

Windows of W recorded steps per sensor over (energy count, flux x, flux y), flux in fixed point
(2^20 units per m/s), each window split into B batches of W/B steps; a window's mean is the mean
of its batch means and its standard error their spread over sqrt(B) (sums about the previous
window's mean); window c agrees with the anchor window j when |m_c - m_j| <= z sqrt(se_c^2 +
se_j^2) for all three, and a window that disagrees becomes the anchor (window 0 is the first);
a sensor's onset is j*W for the first anchor j followed by M agreeing windows; the model's
onset is the largest over the sensors, -1 when any sensor has none."""
import numpy as np


def fixed_point(flux: np.ndarray) -> np.ndarray:
    return np.rint(flux * 1048576.0)


def sensor_onsets(energy: np.ndarray, flux: np.ndarray, window: int, batches: int, z: float, patience: int) -> np.ndarray:
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
            if agree:
                streak += 1
                if streak >= patience:
                    out[s] = anchor_w * window
                    break
            else:
                anchor_mean, anchor_se, anchor_w, streak = mean, se, w, 0
            prev_mean = mean
    return out


def model_onset(per_sensor: np.ndarray) -> int:
    return -1 if np.any(per_sensor < 0) else int(per_sensor.max(initial=-1))
