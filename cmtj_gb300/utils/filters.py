"""`cmtj.utils.filters` (cmtj/utils/filters.py:5-56): the Butterworth
filters the spin-diode post-processing uses, on scipy.signal as in the
reference.  The on-device weighted sum (cmtj_gb300.batch.BatchRun with
red_weights) gives the mean of butter_lowpass_filter without logging the
trajectory."""
import numpy as np
from scipy.signal import butter, lfilter


class Filters:
    @staticmethod
    def butter_bandpass_filter(data, pass_freq, fs, order=5):
        """Band-pass Butterworth filter (filters.py:7-31).  A tuple gives the
        (low, high) band in units of the Nyquist frequency; a float f gives
        the band [0.9 f, f] / Nyquist (f = 0 is taken as 0.1).  The
        reference's float branch designs the filter only for f = 0 (its
        `try` sits inside the `if pass_freq == 0` block); here every float
        is designed."""
        nyq = 0.5 * fs
        if isinstance(pass_freq, tuple):
            b, a = butter(order, [pass_freq[0], pass_freq[1]], btype="bandpass", analog=False)
        else:
            f = 0.1 if pass_freq == 0 else float(pass_freq)
            b, a = butter(order, [0.9 * f / nyq, f / nyq], btype="bandpass", analog=False)
        return lfilter(b, a, data, zi=None)

    @staticmethod
    def butter_lowpass_filter(data, cutoff, fs, order=5):
        """Low-pass Butterworth filter (filters.py:33-43)."""
        b, a = butter(order, cutoff / (0.5 * fs), btype="low", analog=False)
        return lfilter(b, a, data, zi=None)

    @staticmethod
    def detrend_axis(arr, axis):
        """Subtract the median along `axis` (filters.py:45-52)."""
        medians = np.median(arr, axis=axis)
        return (arr.T - medians).T if axis else arr - medians


__all__ = ["Filters"]
