"""BF16 U-Net image-domain network, trained and run by this package's kernels.

The convolutions (forward, weight gradient, data gradient) run on tcgen05
tensor-core GEMMs: 3x3 stride-1 layers as implicit convolutions
(``kgb_conv3x3_bf16``, one halo row per tap row for image rows of 128-pixel
multiples) and implicit weight gradients (``kgb_conv3x3_wgrad_bf16`` on
operands transposed per image row); the stride-2 layers as GEMMs
(``kgb_gemm_bf16_tn`` / ``kgb_gemm_bf16_tn_splitk``) on operands unfolded by
``kgb_unet_unfold`` / ``kgb_unet_unfold_t``, except their data gradient on
rows of 128-pixel multiples, which runs as the four pixel-parity classes of
implicit convolutions (``kgb_conv3x3_s2_dgrad_bf16``).  The two layers with one
channel on a side -- the first 3x3 convolution of the one-channel input and
the 1x1 head to one channel -- are direct kernels (a GEMM would be 1/8 or
1/64 occupied).  ReLU masks, bias gradients, upsampling, skip concatenation,
the MSE loss and Adam are the ``kgb_unet_*`` kernels.  PyTorch only allocates device memory and
provides the stream.  Activations are NHWC bf16 (an image of the Kirchhoff
model, shape (nx, nz) with z fastest, is NHWC with H = nx, W = nz, C = 1);
gradients between layers are float32, master weights and Adam moments
float32.

Topology for ``levels`` = L and ``base`` = c (channels c_l = c 2^l):
encoder level 0: conv3(1->c0)+ReLU, conv3(c0->c0)+ReLU; level l > 0:
conv3 stride 2 (c_{l-1}->c_l)+ReLU, conv3(c_l->c_l)+ReLU; decoder level
l = L-2..0: nearest x2 upsampling of the level-(l+1) output concatenated
with the level-l encoder output, conv3(c_{l+1}+c_l -> c_l)+ReLU,
conv3(c_l->c_l)+ReLU; head conv1(c0 -> 1), linear.

There is no reference counterpart: PyLops has no learned preconditioner.
The oracle for this module is PyTorch CPU autograd on the same weights.
"""

from __future__ import annotations

import math
from typing import Dict, List, Optional

import numpy as np

from .. import _native

__all__ = ["UNet"]


def _rup(n: int, k: int = 8) -> int:
    return (n + k - 1) // k * k


def _halo_weights_fit(C: int, N: int) -> bool:
    """Do the 9-tap weights of an implicit convolution with C input and N
    output channels stay in shared memory next to three halo rows (the
    condition of kgb_conv3x3_s2_dgrad_bf16)?"""
    cblk, bn = (C + 63) // 64, 64 if N <= 64 else 128
    return 1024 + 9 * cblk * bn * 128 + 3 * 18 * 1024 + 8 * 12 + 16 <= 227 * 1024


def _s2_tiles(Hg: int, Wg: int) -> bool:
    """Does a Hg x Wg gradient grid split into 128-pixel tiles for
    kgb_conv3x3_s2_dgrad_bf16 (parts of rows of 128-pixel multiples, or whole
    rows of 32 or 64 pixels)?"""
    return Wg % 128 == 0 or (Wg in (32, 64) and Hg % (128 // Wg) == 0)


def _tileable(H: int, W: int) -> bool:
    """Can 128-pixel M tiles be TMA boxes of one image (kgb_conv3x3_bf16)?"""
    return (W >= 128 and W % 128 == 0) or (W < 128 and 128 % W == 0 and H % (128 // W) == 0)


class _Conv:
    """One convolution layer: shapes, parameter offsets, bf16 weight copies."""

    def __init__(self, cin: int, cout: int, ks: int, stride: int, relu: bool):
        self.cin, self.cout, self.ks, self.stride, self.relu = cin, cout, ks, stride, relu
        self.kc = ks * ks * cin            # real columns of W
        self.kpad = _rup(self.kc)           # padded columns (GEMM K)
        self.kg = _rup(ks * ks * cout)      # data-gradient GEMM K
        self.w_off = 0
        self.b_off = 0
        self.Wb = None                      # bf16 (cout x kpad)
        self.Wt = None                      # bf16 (cin x kg)
        # 3x3 stride-1 convolutions over >= 8 channels also run as implicit
        # GEMMs (kgb_conv3x3_bf16) with weights in 64-channel blocks
        self.implicit = ks == 3 and stride == 1 and cin % 8 == 0
        self.implicit_dx = self.implicit and cout % 8 == 0
        # 3x3 stride-2 layers: data gradient by pixel-parity classes on the
        # tensor cores (kgb_conv3x3_s2_dgrad_bf16) when the gradient rows allow
        self.s2_dx = (ks == 3 and stride == 2 and cout % 8 == 0 and cin % 4 == 0 and cin <= 128
                      and _halo_weights_fit(cout, cin))
        self.Wi = None                      # bf16 (cout x 9 * rup(cin, 64))
        self.Wti = None                     # bf16 (cin x 9 * rup(cout, 64))

    @property
    def nparams(self) -> int:
        return self.cout * self.kpad + self.cout

    def out_hw(self, H: int, W: int):
        p = self.ks // 2
        return (H + 2 * p - self.ks) // self.stride + 1, (W + 2 * p - self.ks) // self.stride + 1


class _CountingLib:
    """The native library with a count of the kernels each entry point
    launches (two for the split-K GEMM, the row sums and the MSE, one for
    the others)."""

    _KERNELS = {"kgb_gemm_bf16_tn_splitk": 2, "kgb_unet_rowsum": 2, "kgb_unet_mse": 2, "kgb_conv3x3_wgrad_bf16": 2,
                "kgb_unet_colsum": 2, "kgb_unet_conv3x3_c1_wgrad": 2,
                "kgb_conv3x3_s2_dgrad_bf16": 4}

    def __init__(self, owner):
        self._owner = owner

    def __getattr__(self, name):
        fn = getattr(_native.lib(), name)
        n = self._KERNELS.get(name, 1)
        owner = self._owner

        def call(*args):
            owner.launches += n
            return fn(*args)

        return call


class UNet:
    """U-Net of ``levels`` levels and ``base`` channels; weights live on the
    current CUDA device.  ``forward(x)`` maps a float32 batch (B, H, W) to
    (B, H, W); ``train_step(x, t)`` does forward, MSE loss, backward and one
    Adam step.  H and W must be divisible by 2^(levels-1) and the number of
    pixels of the coarsest level (B H W / 4^(levels-1)) by 8."""

    def __init__(self, levels: int = 4, base: int = 32, seed: int = 0, normalize: bool = True, implicit: bool = True):
        import torch

        self.implicit = bool(implicit)  # implicit-GEMM 3x3 convolutions where the geometry allows

        if levels < 1:
            raise ValueError("levels must be >= 1")
        self.levels, self.base, self.normalize = levels, base, normalize
        self.ch = [base * 2 ** l for l in range(levels)]
        L = levels
        convs: List[_Conv] = []
        self.enc: List[tuple] = []  # (conv index a, conv index b) per level
        for l in range(L):
            if l == 0:
                convs.append(_Conv(1, self.ch[0], 3, 1, True))
            else:
                convs.append(_Conv(self.ch[l - 1], self.ch[l], 3, 2, True))
            convs.append(_Conv(self.ch[l], self.ch[l], 3, 1, True))
            self.enc.append((len(convs) - 2, len(convs) - 1))
        self.dec: Dict[int, tuple] = {}
        for l in range(L - 2, -1, -1):
            convs.append(_Conv(self.ch[l + 1] + self.ch[l], self.ch[l], 3, 1, True))
            convs.append(_Conv(self.ch[l], self.ch[l], 3, 1, True))
            self.dec[l] = (len(convs) - 2, len(convs) - 1)
        convs.append(_Conv(self.ch[0], 1, 1, 1, False))
        self.head = len(convs) - 1
        self.convs = convs
        # one flat float32 parameter vector: [W (cout x kpad), b (cout)] per layer,
        # each block starting on a 64-element boundary
        off = 0
        for c in convs:
            c.w_off = off
            off = _rup(off + c.cout * c.kpad, 64)
            c.b_off = off
            off = _rup(off + c.cout, 64)
        self.nparams_padded = off
        dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        rng = np.random.default_rng(seed)
        host = np.zeros(off, dtype=np.float32)
        for c in convs:
            std = math.sqrt(2.0 / c.kc) if c.relu else math.sqrt(1.0 / c.kc)
            w = np.zeros((c.cout, c.kpad), dtype=np.float32)
            w[:, :c.kc] = rng.standard_normal((c.cout, c.kc)) * std
            host[c.w_off:c.w_off + w.size] = w.ravel()
        self.params = torch.from_numpy(host).to(dev)
        self.grads = torch.zeros_like(self.params)
        self.adam_m = torch.zeros_like(self.params)
        self.adam_v = torch.zeros_like(self.params)
        self.step_count = 0
        self.launches = 0  # kernels launched by this network so far
        for c in convs:
            c.Wb = torch.empty((c.cout, c.kpad), dtype=torch.bfloat16, device=dev)
            c.Wt = torch.empty((c.cin, c.kg), dtype=torch.bfloat16, device=dev)
            if c.implicit or c.s2_dx:
                c.Wi = torch.empty((c.cout, 9 * _rup(c.cin, 64)), dtype=torch.bfloat16, device=dev)
                if c.implicit_dx or c.s2_dx:
                    c.Wti = torch.empty((c.cin, 9 * _rup(c.cout, 64)), dtype=torch.bfloat16, device=dev)
        self._refresh_weights()
        self._ws = None
        self._ws_key = None
        self._err = torch.zeros(1, dtype=torch.int32, device=dev)
        self._partials = torch.zeros(304, dtype=torch.float64, device=dev)
        self._loss = torch.zeros(1, dtype=torch.float64, device=dev)

    # ------------------------------------------------------------ helpers
    def _lib(self):
        return _CountingLib(self)

    @staticmethod
    def _stream():
        import torch

        return torch.cuda.current_stream().cuda_stream

    def _w(self, c: _Conv):
        return self.params[c.w_off:c.w_off + c.cout * c.kpad]

    def _b(self, c: _Conv):
        return self.params[c.b_off:c.b_off + c.cout]

    def _dw(self, c: _Conv):
        return self.grads[c.w_off:c.w_off + c.cout * c.kpad]

    def _db(self, c: _Conv):
        return self.grads[c.b_off:c.b_off + c.cout]

    def _refresh_weights(self):
        L = self._lib()
        s = self._stream()
        for c in self.convs:
            _native.check(L.kgb_unet_weights(self._w(c).data_ptr(), c.Wb.data_ptr(), c.Wt.data_ptr(), c.cout, c.cin,
                                             c.ks, c.kpad, c.kg, s))
            if c.Wi is not None:
                _native.check(L.kgb_unet_weights_implicit(self._w(c).data_ptr(), c.Wi.data_ptr(),
                                                          c.Wti.data_ptr() if c.Wti is not None else None, c.cout,
                                                          c.cin, c.kpad, s))

    def get_weights(self) -> List[tuple]:
        """Per layer (W (cout, cin, ks, ks), b (cout,)) as float32 numpy arrays
        in the (out, in, kh, kw) convention of ``torch.nn.functional.conv2d``
        on NCHW images."""
        host = self.params.cpu().numpy()
        out = []
        for c in self.convs:
            w = host[c.w_off:c.w_off + c.cout * c.kpad].reshape(c.cout, c.kpad)[:, :c.kc]
            w = w.reshape(c.cout, c.ks, c.ks, c.cin).transpose(0, 3, 1, 2).copy()
            out.append((w, host[c.b_off:c.b_off + c.cout].copy()))
        return out

    def gradients(self) -> List[tuple]:
        host = self.grads.cpu().numpy()
        out = []
        for c in self.convs:
            w = host[c.w_off:c.w_off + c.cout * c.kpad].reshape(c.cout, c.kpad)[:, :c.kc]
            w = w.reshape(c.cout, c.ks, c.ks, c.cin).transpose(0, 3, 1, 2).copy()
            out.append((w, host[c.b_off:c.b_off + c.cout].copy()))
        return out

    def state_dict(self) -> dict:
        return {"levels": self.levels, "base": self.base, "normalize": self.normalize,
                "params": self.params.cpu().numpy().copy(), "step": self.step_count}

    def load_state_dict(self, sd: dict) -> None:
        import torch

        if int(sd["levels"]) != self.levels or int(sd["base"]) != self.base:
            raise ValueError("state dict is for a different topology")
        self.params.copy_(torch.from_numpy(np.asarray(sd["params"], dtype=np.float32)))
        self.normalize = bool(sd.get("normalize", True))
        self.step_count = int(sd.get("step", 0))
        self._refresh_weights()

    def flops(self, H: int, W: int, training: bool = False) -> float:
        """Algorithmic multiply-add flops (2 per MAC) of the convolutions for
        one H x W image: forward, or forward + weight and data gradients."""
        hw = [(H >> l, W >> l) for l in range(self.levels)]
        lvl = {}
        for l, (a, b) in enumerate(self.enc):
            lvl[a] = lvl[b] = l
        for l, (a, b) in self.dec.items():
            lvl[a] = lvl[b] = l
        lvl[self.head] = 0
        total = 0.0
        for i, c in enumerate(self.convs):
            h, w = hw[lvl[i]]
            f = 2.0 * h * w * c.cout * c.kc
            total += f
            if training:
                total += f + (f if i != 0 else 0.0)
        return total

    # ------------------------------------------------------------ buffers
    def _workspace(self, B: int, H: int, W: int):
        import torch

        key = (B, H, W)
        if self._ws_key == key:
            return self._ws
        f = 2 ** (self.levels - 1)
        if H % f or W % f:
            raise ValueError(f"image sides must be multiples of {f}")
        if (B * H * W // f // f) % 8:
            raise ValueError("pixels of the coarsest level (B*H*W/4^(levels-1)) must be a multiple of 8")
        dev = self.device
        bf, f32 = torch.bfloat16, torch.float32
        hw = [(H >> l, W >> l) for l in range(self.levels)]
        P = [B * h * w for h, w in hw]
        ws = {"hw": hw, "P": P}
        ws["x"] = torch.empty(P[0], dtype=bf, device=dev)
        ws["scale"] = torch.empty(B, dtype=f32, device=dev)
        # activation (bf16) and gradient (float32) of every conv output
        lvl_of = {}
        for l, (a, b) in enumerate(self.enc):
            lvl_of[a] = lvl_of[b] = l
        for l, (a, b) in self.dec.items():
            lvl_of[a] = lvl_of[b] = l
        lvl_of[self.head] = 0
        ws["lvl"] = lvl_of
        ws["y"] = [torch.empty(P[lvl_of[i]] * c.cout, dtype=bf if i != self.head else f32, device=dev)
                   for i, c in enumerate(self.convs)]
        ws["dy"] = [torch.empty(P[lvl_of[i]] * c.cout, dtype=f32, device=dev) for i, c in enumerate(self.convs)]
        ws["cat"] = {l: torch.empty(P[l] * (self.ch[l + 1] + self.ch[l]), dtype=bf, device=dev) for l in self.dec}
        ws["dcat"] = {l: torch.empty(P[l] * (self.ch[l + 1] + self.ch[l]), dtype=f32, device=dev) for l in self.dec}
        # unfold / g workspaces sized for the largest layer
        col = gmax = 0
        for i, c in enumerate(self.convs):
            lo = lvl_of[i]
            li = lo - 1 if c.stride == 2 else lo
            col = max(col, P[lo] * c.kpad, P[lo] * c.kc, P[li] * c.kg)
            gmax = max(gmax, P[lo] * c.cout)
        ws["col"] = torch.empty(col, dtype=bf, device=dev)
        ws["g"] = torch.empty(gmax, dtype=bf, device=dev)
        ws["gT"] = torch.empty(gmax, dtype=bf, device=dev)
        ws["gTr"] = torch.empty(gmax, dtype=bf, device=dev)
        ws["work_elems"] = 1 << 23
        ws["work"] = torch.empty(ws["work_elems"], dtype=f32, device=dev)
        self._ws, self._ws_key = ws, key
        return ws

    def _in_of(self, i: int, ws):
        """(input tensor, level of input) of conv i."""
        for l, (a, b) in enumerate(self.enc):
            if i == a:
                return (ws["x"], 0) if l == 0 else (ws["y"][self.enc[l - 1][1]], l - 1)
            if i == b:
                return ws["y"][a], l
        for l, (a, b) in self.dec.items():
            if i == a:
                return ws["cat"][l], l
            if i == b:
                return ws["y"][a], l
        return ws["y"][self.dec[0][1] if self.levels > 1 else self.enc[0][1]], 0

    # ------------------------------------------------------------ layers
    def _conv_forward(self, i: int, ws, B: int):
        c = self.convs[i]
        L, s = self._lib(), self._stream()
        x, li = self._in_of(i, ws)
        lo = ws["lvl"][i]
        (H, W), (Ho, Wo) = ws["hw"][li], ws["hw"][lo]
        P_out = ws["P"][lo]
        if self._is_head1(c):
            # 1x1 convolution to one channel: a dot product per pixel
            _native.check(L.kgb_unet_head_forward(x.data_ptr(), c.Wb.data_ptr(), self._b(c).data_ptr(),
                                                  ws["y"][i].data_ptr(), P_out, c.cin, s))
            return
        if self._is_first1(c):
            # 3x3 convolution of the one-channel input: nine taps per pixel
            _native.check(L.kgb_unet_conv3x3_c1(x.data_ptr(), c.Wb.data_ptr(), self._b(c).data_ptr(),
                                                ws["y"][i].data_ptr(), B, H, W, c.cout, c.kpad, int(c.relu), s))
            return
        if c.ks == 1 and c.stride == 1 and c.cin % 8 == 0:
            A, lda = x, c.cin
        elif self.implicit and c.implicit and _tileable(Ho, Wo):
            A, lda = None, 0
        else:
            A, lda = ws["col"], c.kpad
            _native.check(L.kgb_unet_unfold(x.data_ptr(), A.data_ptr(), B, H, W, c.cin, Ho, Wo, c.ks, c.stride, 0,
                                            c.kpad, s))
        y = ws["y"][i]
        flags = (1 if c.relu else 0) | (2 if i != self.head else 0)
        if self.implicit and c.implicit and _tileable(Ho, Wo):
            _native.check(L.kgb_conv3x3_bf16(x.data_ptr(), c.Wi.data_ptr(), y.data_ptr(), B, H, W, c.cin, c.cout, 0,
                                             self._b(c).data_ptr(), flags, self._err.data_ptr(), s))
            return
        _native.check(L.kgb_gemm_bf16_tn(A.data_ptr(), c.Wb.data_ptr(), y.data_ptr(), P_out, c.cout, c.kpad, lda,
                                         c.kpad, c.cout, self._b(c).data_ptr(), flags, self._err.data_ptr(), s))

    @staticmethod
    def _is_head1(c: _Conv) -> bool:
        return c.ks == 1 and c.stride == 1 and c.cout == 1 and c.cin % 8 == 0 and c.cin <= 256

    @staticmethod
    def _is_first1(c: _Conv) -> bool:
        return c.ks == 3 and c.stride == 1 and c.cin == 1 and c.cout % 8 == 0 and c.cout <= 128

    def _conv_backward(self, i: int, ws, B: int, dx: Optional[object]):
        """Weight/bias gradients of conv i from ws['dy'][i]; data gradient
        into dx (float32, input pixels x cin) unless dx is None."""
        c = self.convs[i]
        L, s = self._lib(), self._stream()
        x, li = self._in_of(i, ws)
        lo = ws["lvl"][i]
        (H, W), (Ho, Wo) = ws["hw"][li], ws["hw"][lo]
        P_in, P_out = ws["P"][li], ws["P"][lo]
        g, gT, col = ws["g"], ws["gT"], ws["col"]
        n = P_out * c.cout
        _native.check(L.kgb_unet_relu_grad(ws["dy"][i].data_ptr(), ws["y"][i].data_ptr() if c.relu else None,
                                           g.data_ptr(), n, int(c.relu), s))
        if self._is_head1(c):
            # head: bias = sum g, weights = g-weighted column sums of x,
            # data gradient g w (no unfolded copies)
            _native.check(L.kgb_unet_rowsum(g.data_ptr(), self._db(c).data_ptr(), 1, P_out, ws["work"].data_ptr(), s))
            _native.check(L.kgb_unet_colsum(x.data_ptr(), g.data_ptr(), self._dw(c).data_ptr(), P_out, c.cin,
                                            ws["work"].data_ptr(), s))
            if dx is not None:
                _native.check(L.kgb_unet_head_dx(g.data_ptr(), c.Wb.data_ptr(), dx.data_ptr(), P_out, c.cin, s))
            return
        if self._is_first1(c) and dx is None:
            _native.check(L.kgb_unet_colsum(g.data_ptr(), None, self._db(c).data_ptr(), P_out, c.cout,
                                            ws["work"].data_ptr(), s))
            _native.check(L.kgb_unet_conv3x3_c1_wgrad(x.data_ptr(), g.data_ptr(), self._dw(c).data_ptr(), B, H, W,
                                                      c.cout, c.kpad, ws["work"].data_ptr(), s))
            return
        implicit_wgrad = (self.implicit and c.ks == 3 and c.stride == 1 and c.cin % 32 == 0 and c.cout % 8 == 0
                          and W % 64 == 0 and c.cout <= 256)
        if implicit_wgrad:
            # bias gradient as column sums of g (no transposed copy needed)
            _native.check(L.kgb_unet_colsum(g.data_ptr(), None, self._db(c).data_ptr(), P_out, c.cout,
                                            ws["work"].data_ptr(), s))
        else:
            if c.cout == 1:
                gT = g
            else:
                _native.check(L.kgb_unet_transpose(g.data_ptr(), gT.data_ptr(), P_out, c.cout, c.cout, P_out, 0, s))
            _native.check(L.kgb_unet_rowsum(gT.data_ptr(), self._db(c).data_ptr(), c.cout, P_out,
                                             ws["work"].data_ptr(), s))
        if implicit_wgrad:
            # implicit weight gradient: x and g transposed per image row (x in
            # three column-shifted copies) instead of the nine-tap unfolded copy
            gTr = ws["gTr"]
            _native.check(L.kgb_unet_row_transpose(x.data_ptr(), col.data_ptr(), B, H, W, c.cin, 3, s))
            _native.check(L.kgb_unet_row_transpose(g.data_ptr(), gTr.data_ptr(), B, H, W, c.cout, 1, s))
            _native.check(L.kgb_conv3x3_wgrad_bf16(col.data_ptr(), gTr.data_ptr(), self._dw(c).data_ptr(), B, H, W,
                                                   c.cin, c.cout, c.kpad, ws["work"].data_ptr(), ws["work_elems"],
                                                   self._err.data_ptr(), s))
        else:
            _native.check(L.kgb_unet_unfold_t(x.data_ptr(), col.data_ptr(), B, H, W, c.cin, c.ks, c.stride, s))
            _native.check(L.kgb_gemm_bf16_tn_splitk(gT.data_ptr(), col.data_ptr(), self._dw(c).data_ptr(), c.cout,
                                                    c.kc, P_out, P_out, P_out, c.kpad, 0, ws["work"].data_ptr(),
                                                    ws["work_elems"], self._err.data_ptr(), s))
        if dx is None:
            return
        if self.implicit and c.implicit_dx and _tileable(H, W):
            # the transposed convolution straight from g (no unfold)
            _native.check(L.kgb_conv3x3_bf16(g.data_ptr(), c.Wti.data_ptr(), dx.data_ptr(), B, H, W, c.cout, c.cin, 1,
                                             None, 0, self._err.data_ptr(), s))
            return
        if self.implicit and c.s2_dx and _s2_tiles(Ho, Wo) and H == 2 * Ho and W == 2 * Wo:
            # stride 2: the four pixel-parity classes straight from g (no unfold)
            _native.check(L.kgb_conv3x3_s2_dgrad_bf16(g.data_ptr(), c.Wti.data_ptr(), dx.data_ptr(), B, Ho, Wo,
                                                      c.cout, c.cin, self._err.data_ptr(), s))
            return
        _native.check(L.kgb_unet_unfold(g.data_ptr(), col.data_ptr(), B, Ho, Wo, c.cout, H, W, c.ks, c.stride, 1,
                                        c.kg, s))
        _native.check(L.kgb_gemm_bf16_tn(col.data_ptr(), c.Wt.data_ptr(), dx.data_ptr(), P_in, c.cin, c.kg, c.kg,
                                         c.kg, c.cin, None, 0, self._err.data_ptr(), s))

    # ------------------------------------------------------------ passes
    def _prepare(self, x):
        import torch

        if x.dim() == 2:
            x = x.unsqueeze(0)
        B, H, W = x.shape
        xx = x.to(device=self.device, dtype=torch.float32).contiguous()
        ws = self._workspace(B, H, W)
        L, s = self._lib(), self._stream()
        if self.normalize:
            _native.check(L.kgb_unet_image_rms(xx.data_ptr(), H * W, B, ws["scale"].data_ptr(), s))
            scale = ws["scale"].data_ptr()
        else:
            scale = None
        _native.check(L.kgb_unet_to_bf16(xx.data_ptr(), ws["x"].data_ptr(), H * W, B, scale, s))
        return ws, B, H, W

    def _forward_all(self, ws, B):
        L, s = self._lib(), self._stream()
        for l, (a, b) in enumerate(self.enc):
            self._conv_forward(a, ws, B)
            self._conv_forward(b, ws, B)
        for l in range(self.levels - 2, -1, -1):
            a, b = self.dec[l]
            cu, ck = self.ch[l + 1], self.ch[l]
            deeper = self.dec[l + 1][1] if (l + 1) in self.dec else self.enc[self.levels - 1][1]
            h, w = ws["hw"][l + 1]
            cat = ws["cat"][l]
            _native.check(L.kgb_unet_upsample(ws["y"][deeper].data_ptr(), cat.data_ptr(), B, h, w, cu, cu + ck, 0, 0,
                                              s))
            _native.check(L.kgb_unet_channels(ws["y"][self.enc[l][1]].data_ptr(), cat.data_ptr(), ws["P"][l], ck,
                                              cu + ck, cu, 0, 0, s))
            self._conv_forward(a, ws, B)
            self._conv_forward(b, ws, B)
        self._conv_forward(self.head, ws, B)

    def forward(self, x):
        """Network output for a float32 batch (B, H, W) or one image (H, W),
        as a float32 CUDA tensor of the same shape (input normalised by its
        RMS per image when ``normalize``)."""
        squeeze = x.dim() == 2
        ws, B, H, W = self._prepare(x)
        self._forward_all(ws, B)
        out = ws["y"][self.head].view(B, H, W).clone()
        return out[0] if squeeze else out

    __call__ = forward

    def backward_from(self, ws, B):
        """All parameter gradients from ws['dy'][head] (float32)."""
        L, s = self._lib(), self._stream()
        dec_first = self.dec[0][1] if self.levels > 1 else self.enc[0][1]
        self._conv_backward(self.head, ws, B, ws["dy"][dec_first])
        pending = {}
        for l in range(0, self.levels - 1):
            a, b = self.dec[l]
            self._conv_backward(b, ws, B, ws["dy"][a])
            self._conv_backward(a, ws, B, ws["dcat"][l])
            cu, ck = self.ch[l + 1], self.ch[l]
            deeper = self.dec[l + 1][1] if (l + 1) in self.dec else self.enc[self.levels - 1][1]
            h, w = ws["hw"][l + 1]
            _native.check(L.kgb_unet_upsample(ws["dcat"][l].data_ptr(), ws["dy"][deeper].data_ptr(), B, h, w, cu,
                                              cu + ck, 0, 1, s))
            pending[l] = (ws["dcat"][l], cu, ck)
        for l in range(self.levels - 1, -1, -1):
            a, b = self.enc[l]
            self._conv_backward(b, ws, B, ws["dy"][a])
            below = ws["dy"][self.enc[l - 1][1]] if l > 0 else None
            self._conv_backward(a, ws, B, below)
            if l > 0 and (l - 1) in pending:
                # the level-(l-1) encoder output also feeds the decoder concatenation
                dcat, cu, ck = pending[l - 1]
                _native.check(L.kgb_unet_channels(dcat.data_ptr(), below.data_ptr(), ws["P"][l - 1], ck, cu + ck,
                                                  cu, 1, 1, s))
        if self.levels == 1:
            return

    def loss_and_grad(self, x, t):
        """Forward, MSE loss against float32 targets t (same shape as x) and
        backward; returns the loss as a 0-d float64 CUDA tensor.  Targets are
        compared with the raw network output (the input normalisation does
        not rescale them)."""
        import torch

        ws, B, H, W = self._prepare(x)
        self._forward_all(ws, B)
        tt = t.to(device=self.device, dtype=torch.float32).contiguous()
        L, s = self._lib(), self._stream()
        n = B * H * W
        _native.check(L.kgb_unet_mse(ws["y"][self.head].data_ptr(), tt.data_ptr(), ws["dy"][self.head].data_ptr(),
                                     n, self._partials.data_ptr(), self._loss.data_ptr(), s))
        self.backward_from(ws, B)
        return self._loss[0]

    def adam_step(self, lr: float = 1e-3, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8) -> None:
        L, s = self._lib(), self._stream()
        self.step_count += 1
        _native.check(L.kgb_unet_adam(self.params.data_ptr(), self.grads.data_ptr(), self.adam_m.data_ptr(),
                                      self.adam_v.data_ptr(), self.nparams_padded, lr, b1, b2, eps, self.step_count,
                                      s))
        self._refresh_weights()

    def train_step(self, x, t, lr: float = 1e-3):
        loss = self.loss_and_grad(x, t)
        self.adam_step(lr)
        return loss

    def check_errors(self) -> None:
        """Raise if a GEMM pipeline wait timed out since the last check."""
        if int(self._err.item()):
            self._err.zero_()
            raise RuntimeError("tensor-core GEMM pipeline wait timed out")
