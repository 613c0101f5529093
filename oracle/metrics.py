"""CPU restatement of the reference's image metrics (test infrastructure only).

CalculateMSE and CalculateRMAE (mse.cpp:33-65): per pixel the float3 difference, its
square (MSE) or absolute value (MAE), the three channels summed in float, the pixel
sums accumulated in double, divided by 3 * pixel count.
"""
import numpy as np


def mse_mae(gt_rgb, img_rgb):
    gt = np.asarray(gt_rgb, np.float32).reshape(-1, 3)
    x = np.asarray(img_rgb, np.float32).reshape(-1, 4)[:, :3] if np.asarray(img_rgb).shape[-1] == 4 \
        else np.asarray(img_rgb, np.float32).reshape(-1, 3)
    d = (gt - x).astype(np.float32)
    sq = (d * d).astype(np.float32)
    s3 = ((sq[:, 0] + sq[:, 1]).astype(np.float32) + sq[:, 2]).astype(np.float32)
    ad = np.abs(d)
    a3 = ((ad[:, 0] + ad[:, 1]).astype(np.float32) + ad[:, 2]).astype(np.float32)
    n = gt.shape[0]
    return float(np.sum(s3.astype(np.float64)) / (n * 3)), float(np.sum(a3.astype(np.float64)) / (n * 3))
