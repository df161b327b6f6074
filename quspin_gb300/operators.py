"""Quantum operators on the GPU: ``hamiltonian`` and ``quantum_LinearOperator``.

Drop-in counterparts of QuSpin 1.0.1's

* ``hamiltonian`` (src/quspin/operators/hamiltonian_core.py:187): the
  constructor builds the static CSR/DIA and the ``{function: matrix}``
  dynamic parts (:221-500 with _make_hamiltonian.py:19-133) on the GPU;
  ``dot`` (:615-788) applies them with the kernels of ``csrc/sparse.cu``;
  ``tocsr`` (:1686-1720) returns the host scipy matrix.
* ``quantum_LinearOperator`` (src/quspin/operators/quantum_LinearOperator_core.py:25):
  the matrix-free apply, diagonal part stored at construction (:143-155) and
  the off-diagonal terms applied by the on-device ``inplace_op`` kernel
  (``dot`` :288-347, ``_matvec`` :520-540).

Operands may be numpy arrays (copied to the device and back, as a user of
the reference passes them) or CUDA torch tensors (kept on the device).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from . import _device as D
from . import _lib
from .basis import _TermTable, basis_general, build_matrix, spin_basis_1d
from .sparse import DeviceCSR, DeviceDIA, result_dtype, to_device_matrix

supported_dtypes = tuple(D.SUPPORTED)


def _consolidate_static(static_list):
    """Merge repeated (opstr, sites) bonds, drop |J| <= 10 eps (_make_hamiltonian.py:19-41)."""
    eps = 10 * np.finfo(np.float64).eps
    d = {}
    for opstr, bonds in static_list:
        dd = d.setdefault(opstr, {})
        for bond in bonds:
            J = bond[0]
            indx = tuple(bond[1:])
            dd[indx] = dd[indx] + J if indx in dd else J
    out = []
    for opstr, dd in d.items():
        for indx, J in dd.items():
            if np.abs(J) > eps:
                out.append((opstr, indx, J))
    return out


def _consolidate_dynamic(dynamic_list):
    """Group dynamic bonds by (function, args) (_make_hamiltonian.py:44-71)."""
    eps = 10 * np.finfo(np.float64).eps
    d = {}
    for opstr, bonds, f, f_args in dynamic_list:
        key = (opstr, f, tuple(f_args))
        dd = d.setdefault(key, {})
        for bond in bonds:
            J = bond[0]
            indx = tuple(bond[1:])
            dd[indx] = dd[indx] + J if indx in dd else J
    out = {}
    for (opstr, f, f_args), dd in d.items():
        out.setdefault((f, f_args), []).extend(
            [(opstr, indx, J) for indx, J in dd.items() if np.abs(J) > eps])
    return out


class function:
    """Time-dependent coefficient f(t, *args) (src/quspin/operators/_functions.py:1-47)."""

    def __init__(self, func, args):
        self._func = func
        self._args = tuple(args)

    def __call__(self, *t):
        return self._func(*t, *self._args)

    def __hash__(self):
        return hash((self._func, self._args))

    def __eq__(self, other):
        return isinstance(other, function) and self._func == other._func and self._args == other._args

    def __repr__(self):
        return "function({}, {})".format(getattr(self._func, "__name__", self._func), self._args)


def _is_opstr_entry(e):
    return isinstance(e, (list, tuple)) and len(e) >= 2 and isinstance(e[0], str)


def ishamiltonian(x):
    return isinstance(x, hamiltonian)


class hamiltonian:
    """Static + time-dependent operator built on the GPU (hamiltonian_core.py:187)."""

    def __init__(self, static_list, dynamic_list, N=None, basis=None, shape=None, dtype=np.complex128,
                 static_fmt=None, dynamic_fmt=None, copy=True, check_symm=True, check_herm=True,
                 check_pcon=True, **basis_kwargs):
        dtype = np.dtype(dtype)
        if dtype not in supported_dtypes:
            raise TypeError("hamiltonian does not support type: " + str(dtype))
        self._dtype = dtype
        self._basis = basis
        if type(static_list) not in (list, tuple):
            raise TypeError("expecting list/tuple of lists/tuples containing opstr and list of indx")
        if type(dynamic_list) not in (list, tuple):
            raise TypeError("expecting list/tuple of lists/tuples containing opstr and list of indx, "
                            "functions, and function args")
        static_opstr = [e for e in static_list if _is_opstr_entry(e)]
        static_other = [e for e in static_list if not _is_opstr_entry(e)]
        dynamic_opstr = [e for e in dynamic_list if _is_opstr_entry(e)]
        dynamic_other = [e for e in dynamic_list if not _is_opstr_entry(e)]
        self._static_opstr_list = static_opstr
        self._dynamic_opstr_list = dynamic_opstr
        if static_opstr or dynamic_opstr:
            if self._basis is not None:
                if basis_kwargs:
                    raise ValueError("unexpected optional argument(s): " + ", ".join(basis_kwargs))
            else:
                if N is None:
                    raise Exception("if opstrs in use, argument N needed for basis class")
                if type(N) is not int:
                    raise TypeError("argument N must be integer")
                self._basis = spin_basis_1d(N, **basis_kwargs)
            if not isinstance(self._basis, basis_general):
                raise TypeError("expecting instance of basis class for argument: basis")
            Ns = self._basis.Ns
            self._shape = (Ns, Ns)
        else:
            if shape is None:
                mats = [e for e in static_other] + [e[0] for e in dynamic_other]
                if not mats:
                    raise ValueError("missing argument shape")
                shape = mats[0].shape
            self._shape = tuple(shape)
        self._static = None
        if static_opstr:
            self._static = build_matrix(self._basis, _consolidate_static(static_opstr), dtype)
        for M in static_other:
            Md = to_device_matrix(M if not isinstance(M, np.ndarray) else sp.csr_matrix(M), dtype)
            self._static = Md if self._static is None else _add_device(self._static, Md, dtype)
        if self._static is None:
            self._static = DeviceDIA(D.to_device(np.zeros(0, np.int64)),
                                     D.zeros((0, self._shape[0]), dtype), self._shape, dtype)
        self._dynamic = {}
        if dynamic_opstr:
            for (f, f_args), ops in _consolidate_dynamic(dynamic_opstr).items():
                if np.isscalar(f_args):
                    raise TypeError("function arguments must be array type")
                Hd = build_matrix(self._basis, ops, dtype)
                fn = function(f, f_args)
                if Hd.nnz > 0:
                    self._dynamic[fn] = Hd if fn not in self._dynamic else _add_device(self._dynamic[fn], Hd, dtype)
        for e in dynamic_other:
            M, f, f_args = e[0], e[1], e[2]
            Md = to_device_matrix(M if not isinstance(M, np.ndarray) else sp.csr_matrix(M), dtype)
            fn = function(f, f_args)
            self._dynamic[fn] = Md if fn not in self._dynamic else _add_device(self._dynamic[fn], Md, dtype)
        self._union = None

    # -- attributes ---------------------------------------------------------
    @property
    def basis(self):
        if self._basis is None:
            raise ValueError("no basis for this hamiltonian")
        return self._basis

    @property
    def Ns(self):
        return self._shape[0]

    @property
    def shape(self):
        return self._shape

    @property
    def get_shape(self):
        return self._shape

    @property
    def dtype(self):
        return self._dtype

    @property
    def ndim(self):
        return 2

    @property
    def is_dense(self):
        return False

    @property
    def static(self):
        """Static part (device matrix; ``.tocsr()`` gives the scipy copy)."""
        return self._static

    @property
    def dynamic(self):
        return dict(self._dynamic)

    # -- products -------------------------------------------------------------
    def dot(self, V, time=0, check=True, out=None, overwrite_out=True, a=1.0):
        """a H(time) V (hamiltonian_core.py:615-788)."""
        if ishamiltonian(V):
            raise NotImplementedError("operator algebra between hamiltonians is not part of the GPU path")
        times = np.array(time)
        host = not D.is_device_array(V)
        if host:
            V = np.asanyarray(V)
        if check:
            if V.shape[0] != self._shape[1]:
                raise ValueError("matrix dimension mismatch with shapes: {0} and {1}.".format(V.shape, self._shape))
            if V.ndim > 3:
                raise ValueError("Expecting V.ndim < 4.")
        vdt = V.dtype if host else D.np_dtype(V.dtype)
        rdt = result_dtype(vdt, self._dtype)
        if rdt not in supported_dtypes:
            raise TypeError("resulting dtype is not supported.")
        if np.iscomplexobj(a) and rdt.kind != "c":
            rdt = result_dtype(rdt, np.complex64)
        if times.ndim > 0:
            if times.ndim > 1:
                raise ValueError("Expecting time to be one dimensional array-like.")
            if V.shape[-1] != times.shape[0]:
                raise ValueError("For non-scalar times V.shape[-1] must be equal to len(time).")
            cols = []
            for i, t in enumerate(times):
                cols.append(self.dot(V[..., i], time=t, check=False, a=a))
            if host:
                return np.stack(cols, axis=-1)
            return torch.stack(cols, dim=-1)
        x = D.to_device(V, rdt)
        if x.dim() == 3:
            x2 = x.reshape(x.shape[0], -1)
        else:
            x2 = x
        if out is not None:
            odt = np.asarray(out).dtype if not D.is_device_array(out) else D.np_dtype(out.dtype)
            if odt != rdt:
                raise TypeError("'out' must be array with correct dtype and dimensions for output array.")
            if tuple(out.shape) != tuple(V.shape):
                raise ValueError("'out' must be array with correct dtype and dimensions for output array.")
            y = out if D.is_device_array(out) else D.to_device(out, rdt)
            y2 = y.reshape(x2.shape)
        else:
            y = torch.empty_like(x)
            y2 = y.reshape(x2.shape)
            overwrite_out = True
        self._static.matvec_into(x2, y2, a=a, overwrite=overwrite_out)
        for fn, Hd in self._dynamic.items():
            Hd.matvec_into(x2, y2, a=a * fn(time), overwrite=False)
        if host:
            res = D.to_host(y)
            if out is not None:
                out[...] = res
                return out
            return res
        if out is not None and y.data_ptr() != out.data_ptr():
            out.copy_(y)
            return out
        return y

    def __mul__(self, other):
        return self.dot(other)

    def __matmul__(self, other):
        return self.dot(other)

    # -- conversions ------------------------------------------------------------
    def tocsr(self, time=0):
        """Host scipy CSR of H(time) (hamiltonian_core.py:1686-1720)."""
        H = self._static.tocsr().astype(self._dtype)
        for fn, Hd in self._dynamic.items():
            H = H + fn(time) * Hd.tocsr()
        return sp.csr_matrix(H, dtype=self._dtype)

    def toarray(self, time=0):
        return self.tocsr(time).toarray()

    def todense(self, time=0):
        return self.tocsr(time).todense()

    def evolve(self, v0, t0, times, eom="SE", solver_name="dop853", stack_state=False, verbose=False,
               iterate=False, imag_time=False, **solver_args):
        """(Imaginary-)time Schroedinger evolution (hamiltonian_core.py:1489-1630),
        integrated by DOP853 on the device (tools/evolution.py)."""
        from .tools.evolution import evolve_hamiltonian
        return evolve_hamiltonian(self, v0, t0, times, eom=eom, solver_name=solver_name, stack_state=stack_state,
                                  verbose=verbose, iterate=iterate, imag_time=imag_time, **solver_args)

    def tocsr_gpu(self, time=0):
        """Device CSR of H(time).  The union sparsity pattern of the static and
        dynamic parts is built once; each call forms the values on the device."""
        if not self._dynamic:
            if isinstance(self._static, DeviceCSR):
                return self._static
            if self._union is None:
                self._union = DeviceCSR.from_scipy(self._static.tocsr(), self._dtype)
            return self._union
        if self._union is None:
            parts = [sp.csr_matrix(p) for p in
                     [self._static.tocsr()] + [Hd.tocsr() for Hd in self._dynamic.values()]]

            def ones(p):
                return sp.csr_matrix((np.ones(p.nnz), p.indices, p.indptr), shape=p.shape)
            pat = ones(parts[0])
            for p in parts[1:]:
                pat = pat + ones(p)
            pat = sp.csr_matrix(pat)
            pat.sort_indices()
            vals = []
            for p in parts:
                # values of p on the union pattern
                pp = sp.csr_matrix(p, dtype=self._dtype)
                m = pat.copy().astype(self._dtype)
                m.data[:] = 0
                m = m + pp
                m = sp.csr_matrix((np.asarray(m[pat.nonzero()]).ravel(), pat.indices, pat.indptr),
                                  shape=pat.shape)
                vals.append(D.to_device(np.ascontiguousarray(m.data, dtype=self._dtype)))
            base = DeviceCSR.from_scipy(pat.astype(self._dtype), self._dtype)
            self._union = (base, vals, list(self._dynamic.keys()))
        base, vals, fns = self._union
        data = vals[0].clone()
        for v, fn in zip(vals[1:], fns):
            data.add_(v, alpha=complex(fn(time)) if self._dtype.kind == "c" else float(np.real(fn(time))))
        return DeviceCSR(base.indptr, base.indices, data, base.shape, self._dtype)

    def aslinearoperator(self, time=0):
        from scipy.sparse.linalg import LinearOperator
        return LinearOperator(self._shape, dtype=self._dtype, matvec=lambda v: self.dot(v, time=time),
                              matmat=lambda v: self.dot(v, time=time))

    def eigsh(self, time=0, **eigsh_args):
        """scipy ARPACK driven by the GPU product."""
        from scipy.sparse.linalg import eigsh
        return eigsh(self.aslinearoperator(time), **eigsh_args)

    def __repr__(self):
        return "<hamiltonian {} dtype={} static={} dynamic={}>".format(self._shape, self._dtype,
                                                                     self._static.format, len(self._dynamic))


def _add_device(A, B, dtype):
    """Sum of two device matrices (through the host; construction time only)."""
    return DeviceCSR.from_scipy((A.tocsr() + B.tocsr()).astype(dtype), dtype)


class quantum_LinearOperator:
    """Matrix-free operator (quantum_LinearOperator_core.py:25-155, :288-347, :520-540).

    Diagonal terms are summed into a device vector at construction; the other
    terms are applied on every product by the on-device inplace_op kernel
    (representative + index search per element, no stored matrix).
    """

    def __init__(self, operator_list, basis=None, dtype=np.complex128, diagonal=None, check_symm=True,
                 check_herm=True, check_pcon=True, copy=True, **basis_args):
        dtype = np.dtype(dtype)
        if dtype not in supported_dtypes:
            raise TypeError("hamiltonian does not support type: " + str(dtype))
        if basis is None:
            N = basis_args.pop("N", None)
            if N is None:
                raise ValueError("missing basis or argument N")
            basis = spin_basis_1d(N, **basis_args)
        self._basis = basis
        self._dtype = dtype
        self._shape = (basis.Ns, basis.Ns)
        self._transposed = False
        self._conjugated = False
        self._public_static_list = list(operator_list)
        static = _consolidate_static(operator_list)
        diag_terms, self._static_list = [], []
        for opstr, indx, J in static:
            o, _, _ = basis._term(opstr, indx, J)
            (diag_terms if set(o) <= set("Izn") else self._static_list).append((opstr, indx, J))
        self._diagonal = None
        if diagonal is not None:
            self.set_diagonal(diagonal, copy=copy)
        if diag_terms and basis.Ns:
            dm = build_matrix(basis, diag_terms, dtype)
            if dm.nnz:
                d = dm.data.reshape(-1)
                self._diagonal = d if self._diagonal is None else self._diagonal + d
        self._tt = _TermTable([basis._term(o, ix, J) for o, ix, J in self._static_list])

    def set_diagonal(self, diagonal, copy=True):
        d = D.to_device(diagonal)
        if d.dim() != 1 or d.shape[0] != self._shape[0]:
            raise ValueError("diagonal must be a 1-d array of length Ns")
        self._diagonal = d.clone() if copy else d

    @property
    def basis(self):
        return self._basis

    @property
    def shape(self):
        return self._shape

    @property
    def Ns(self):
        return self._shape[0]

    @property
    def dtype(self):
        return self._dtype

    @property
    def diagonal(self):
        return None if self._diagonal is None else D.to_host(self._diagonal)

    @property
    def T(self):
        return self.transpose()

    @property
    def H(self):
        return self.getH()

    def transpose(self, copy=False):
        new = _copy_op(self)
        new._transposed = not self._transposed
        return new

    def conj(self):
        new = _copy_op(self)
        new._conjugated = not self._conjugated
        if new._diagonal is not None and np.dtype(self._dtype).kind == "c":
            new._diagonal = new._diagonal.conj()
        return new

    def getH(self, copy=False):
        return self.conj().transpose()

    def _apply(self, x, y, a):
        """y += a * offdiag(x): device (Ns, k) complex128 blocks."""
        if self._tt.T == 0 or self.Ns == 0:
            return
        err = D.err_flag()
        a = complex(a)
        b = self._basis
        # The reference passes (conjugated, transposed) into the (transposed,
        # conjugated) positions of inplace_Op (quantum_LinearOperator_core.py:335-343);
        # kept as is for identical results.
        _lib.call("qs_inplace_op", b._sym, *b._basis_args(), *self._tt.args(), self._tt.T,
                  int(self._conjugated), int(self._transposed), a.real, a.imag, D.ptr(x), D.ptr(y), x.shape[1],
                  D.ptr(err), D.stream())

    def _product(self, other, out, a, diag_scaled):
        host = not D.is_device_array(other)
        vdt = np.asarray(other).dtype if host else D.np_dtype(other.dtype)
        rdt = result_dtype(self._dtype, vdt)
        shape = tuple(other.shape)
        if shape[0] != self.Ns:
            raise ValueError("dimension mismatch")
        x = D.to_device(other, np.complex128).reshape(self.Ns, -1).contiguous()
        y = torch.zeros_like(x)
        if self._diagonal is not None:
            dg = self._diagonal.to(torch.complex128).reshape(-1, 1)
            y += (dg * x) * (complex(a) if diag_scaled else 1.0)
        self._apply(x, y, a)
        if rdt.kind != "c":
            y = y.real
        y = y.to(D.torch_dtype(rdt)).reshape(shape)
        if out is not None:
            odt = np.asarray(out).dtype if not D.is_device_array(out) else D.np_dtype(out.dtype)
            if (odt, tuple(out.shape)) != (rdt, shape):
                raise ValueError("out must be C-congituous writable array with dtype {} and shape {}.".format(
                    rdt, shape))
            if D.is_device_array(out):
                out.copy_(y)
            else:
                out[...] = D.to_host(y)
            return out
        return D.to_host(y) if host else y

    def dot(self, other, out=None, a=1.0):
        """a H other.  With ``out`` given, the diagonal part is not scaled by
        ``a`` -- the reference's behaviour (quantum_LinearOperator_core.py:323-343)."""
        return self._product(other, out, a, diag_scaled=out is None)

    def matvec(self, other):
        return self._product(other, None, 1.0, True)

    def __mul__(self, other):
        return self.dot(other)

    def __matmul__(self, other):
        return self.dot(other)

    def aslinearoperator(self):
        from scipy.sparse.linalg import LinearOperator
        return LinearOperator(self._shape, dtype=self._dtype, matvec=self.matvec, matmat=self.matvec)


def _copy_op(op):
    new = quantum_LinearOperator.__new__(quantum_LinearOperator)
    new.__dict__.update(op.__dict__)
    return new
