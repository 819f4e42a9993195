"""The GB300 library as a backend for tests/kat_cases.py: every call goes
through the package's reference-shaped API and the C ABI."""
import numpy as np


class GpuBackend:
    def __init__(self, ifx, dtype=np.float64):
        self.ifx = ifx
        self.dtype = dtype

    def _border(self, style, fill):
        return self.ifx.Fill(fill) if style == "fill" else self.ifx.Pad(style)

    def _img(self, a):
        return np.asfortranarray(np.asarray(a, dtype=self.dtype))

    def padarray(self, A, style, lo, hi, fill=0.0):
        ifx = self.ifx
        b = ifx.Fill(fill, tuple(lo), tuple(hi)) if style == "fill" else ifx.Pad(style, tuple(lo), tuple(hi))
        out, _ = ifx.padarray(self._img(A), b)
        return np.asarray(out, dtype=np.float64)

    def cascade(self, img, factors, style, fill=0.0):
        ifx = self.ifx
        img = self._img(img)
        ks = tuple(ifx.ReshapedOneD(ifx.OffsetKernel(np.asarray(w, np.float64), (first,)), img.ndim, ax)
                   for ax, first, w in factors)
        return np.asarray(ifx.imfilter(img, ks, self._border(style, fill)), dtype=np.float64)

    def dense(self, img, K, kfirst, style, fill=0.0):
        ifx = self.ifx
        img = self._img(img)
        k = ifx.OffsetKernel(np.asarray(K, np.float64), tuple(kfirst))
        return np.asarray(ifx.imfilter(img, (k,), self._border(style, fill)), dtype=np.float64)

    def _iir_kern(self, sigmas, nd):
        ifx = self.ifx
        return tuple(ifx.ReshapedOneD(ifx.KernelFactors.IIRGaussian(s), nd, ax) for ax, s in sigmas)

    def iir(self, img, sigmas, style, fill=0.0):
        ifx = self.ifx
        img = self._img(img)
        try:
            out = ifx.imfilter(img, self._iir_kern(sigmas, img.ndim), self._border(style, fill))
        except ifx.DimensionMismatch as e:
            raise ValueError("DimensionMismatch: %s" % e)
        return np.asarray(out, dtype=np.float64)

    def iir_dim(self, img, sigma, dim, style):
        ifx = self.ifx
        img = self._img(img)
        out = np.asfortranarray(np.zeros(img.shape))
        ifx.imfilter_(out, img, ifx.KernelFactors.IIRGaussian(sigma), dim, style)
        return out

    def mixed(self, img, spec, style, fill=0.0):
        ifx = self.ifx
        img = self._img(img)
        nd = img.ndim
        ks = []
        for st in spec:
            if st[0] == "iir":
                ts = ifx.KernelFactors.IIRGaussian(st[2])
                ks.append(ts if nd == 1 else ifx.ReshapedOneD(ts, nd, st[1]))
            elif st[0] == "lap":
                ks.append(ifx.Kernel.Laplacian((True,) * nd))
            else:
                ks.append(ifx.OffsetKernel(np.asarray(st[1], np.float64), tuple(st[2])))
        return np.asarray(ifx.imfilter(img, tuple(ks), self._border(style, fill)), dtype=np.float64)

    def iir_na(self, img, sigmas, na="isnan"):
        ifx = self.ifx
        img = self._img(img)
        return np.asarray(ifx.imfilter(img, self._iir_kern(sigmas, img.ndim), ifx.NA(na)), dtype=np.float64)

    def fft(self, img, K, kfirst, style, fill=0.0):
        ifx = self.ifx
        k = ifx.OffsetKernel(np.asarray(K, np.float64), tuple(kfirst))
        return np.asarray(ifx.imfilter(self._img(img), (k,), self._border(style, fill), ifx.Algorithm.FFT()),
                          dtype=np.float64)

    def fft_cascade(self, img, factors, style, fill=0.0):
        ifx = self.ifx
        img = self._img(img)
        ks = tuple(ifx.ReshapedOneD(ifx.OffsetKernel(np.asarray(w, np.float64), (first,)), img.ndim, ax)
                   for ax, first, w in factors)
        return np.asarray(ifx.imfilter(img, ks, self._border(style, fill), ifx.Algorithm.FFT()),
                          dtype=np.float64)

    def fft_nopad(self, img, K, kfirst):
        ifx = self.ifx
        img = self._img(img)
        out = np.asfortranarray(np.zeros(img.shape))
        k = ifx.OffsetKernel(np.asarray(K, np.float64), tuple(kfirst))
        ifx.imfilter_(out, img, (k,), ifx.NoPad(), ifx.Algorithm.FFT())
        return out

    def laplacian(self, img, flags, style, fill=0.0, arith="f64"):
        ifx = self.ifx
        dt = {"f64": np.float64, "f32": np.float32, "int": np.uint8}[arith]
        a = np.asfortranarray(np.asarray(img, dtype=dt))
        out = ifx.imfilter(a, ifx.Kernel.Laplacian(tuple(bool(f) for f in flags)),
                           self._border(style, fill))
        return np.asarray(out, dtype=np.float64)

    def median(self, img, wf, wl, style, fill=0.0):
        ifx = self.ifx
        win = tuple(range(f, f + l) for f, l in zip(wf, wl))
        return np.asarray(ifx.mapwindow(ifx.median, self._img(img), win, border=self._border(style, fill)),
                          dtype=np.float64)

    def extrema(self, img, wf, wl, style, fill=0.0):
        ifx = self.ifx
        win = tuple(range(f, f + l) for f, l in zip(wf, wl))
        out = ifx.mapwindow(ifx.extrema, self._img(img), win, border=self._border(style, fill))
        return np.asarray(out[0], np.float64), np.asarray(out[1], np.float64)

    def extrema_lemire(self, img, w):
        ifx = self.ifx
        out = ifx.mapwindow(ifx.extrema, self._img(img), tuple(int(x) for x in w))
        return np.asarray(out[0], np.float64), np.asarray(out[1], np.float64)

    def na_cascade(self, img, factors, na="isnan"):
        ifx = self.ifx
        img = self._img(img)
        ks = tuple(ifx.ReshapedOneD(ifx.OffsetKernel(np.asarray(w, np.float64), (first,)), img.ndim, ax)
                   for ax, first, w in factors)
        return np.asarray(ifx.imfilter(img, ks, ifx.NA(na)), dtype=np.float64)

    def na_dense(self, img, K, kfirst, na="isnan"):
        ifx = self.ifx
        img = self._img(img)
        k = ifx.OffsetKernel(np.asarray(K, np.float64), tuple(kfirst))
        return np.asarray(ifx.imfilter(img, (k,), ifx.NA(na)), dtype=np.float64)

    def inner_dense(self, img, K, kfirst):
        ifx = self.ifx
        k = ifx.OffsetKernel(np.asarray(K, np.float64), tuple(kfirst))
        out = ifx.imfilter(self._img(img), (k,), ifx.Inner())
        return np.asarray(out, dtype=np.float64), out.first

    def inner_cascade(self, img, factors):
        ifx = self.ifx
        img = self._img(img)
        ks = tuple(ifx.ReshapedOneD(ifx.OffsetKernel(np.asarray(w, np.float64), (first,)), img.ndim, ax)
                   for ax, first, w in factors)
        out = ifx.imfilter(img, ks, ifx.Inner())
        return np.asarray(out, dtype=np.float64), out.first

    def localextrema(self, img, window=None, edges=True, minima=False):
        ifx = self.ifx
        f = ifx.findlocalminima if minima else ifx.findlocalmaxima
        return f(self._img(img), window=window, edges=edges)

    def blob_log(self, img, sigmas, edges=None, sigma_shape=None, rthresh=0.001):
        ifx = self.ifx
        bl = ifx.blob_LoG(self._img(img), sigmas, edges=edges, sigma_shape=sigma_shape, rthresh=rthresh)
        return [(b.location, b.sigma, b.amplitude) for b in bl]
