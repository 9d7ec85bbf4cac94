"""``ot.utils`` pieces on the path: ``dist`` for the squared-Euclidean and
Euclidean metrics (``ot/utils.py:400``), and the result container
``OTResult`` (``ot/utils.py:1127``) with the fields the solvers fill
(``plan``, ``value``, ``value_linear``, ``potentials``, ``log``, ``lazy_plan``)
and the derived properties users read from them."""


def dist(x1, x2=None, metric="sqeuclidean", p=2, w=None, backend="auto", nx=None, use_tensor=False):
    """GPU ``ot.dist`` for 'sqeuclidean' and 'euclidean' (``ot/utils.py:400-470``):
    the cost kernel of the batch path with one problem.  ``x2=None`` means
    ``x2 = x1`` (zero diagonal); other metrics raise NotImplementedError."""
    from . import batch as pb
    X1 = x1[None] if hasattr(x1, "shape") else [x1]
    X2 = None if x2 is None else (x2[None] if hasattr(x2, "shape") else [x2])
    M = pb.dist_batch(X1, X2, metric=metric, p=p)
    return M[0]


class OTResult:
    def __init__(self, potentials=None, value=None, value_linear=None, value_quad=None, plan=None,
                 log=None, backend=None, sparse_plan=None, lazy_plan=None, status=None, batch_size=0):
        self._potentials = potentials
        self._value = value
        self._value_linear = value_linear
        self._value_quad = value_quad
        self._plan = plan
        self._log = log
        self._sparse_plan = sparse_plan
        self._lazy_plan = lazy_plan
        self._backend = backend
        self._status = status
        self._batch_size = batch_size

    def __repr__(self):
        s = "OTResult("
        if self._value is not None:
            s += "value={},".format(self._value)
        if self._value_linear is not None:
            s += "value_linear={},".format(self._value_linear)
        if self._plan is not None:
            s += "plan={}(shape={}),".format(self._plan.__class__.__name__, tuple(self._plan.shape))
        if s[-1] != "(":
            s = s[:-1] + ")"
        else:
            s = s + ")"
        return s

    @property
    def potentials(self):
        return self._potentials

    @property
    def potential_a(self):
        return None if self._potentials is None else self._potentials[0]

    @property
    def potential_b(self):
        return None if self._potentials is None else self._potentials[1]

    @property
    def value(self):
        return self._value

    @property
    def value_linear(self):
        return self._value_linear

    @property
    def value_quad(self):
        return self._value_quad

    @property
    def plan(self):
        return self._plan

    @property
    def lazy_plan(self):
        return self._lazy_plan

    @property
    def sparse_plan(self):
        return self._sparse_plan

    @property
    def log(self):
        return self._log

    @property
    def status(self):
        return self._status

    @property
    def marginals(self):
        return self.marginal_a, self.marginal_b

    @property
    def marginal_a(self):
        if self._plan is None:
            return None
        return self._plan.sum(-1)

    @property
    def marginal_b(self):
        if self._plan is None:
            return None
        return self._plan.sum(-2)

    @property
    def a_to_b(self):
        raise NotImplementedError()

    @property
    def b_to_a(self):
        raise NotImplementedError()

    @property
    def citation(self):
        return ("Flamary R., Courty N., Gramfort A., et al., POT Python Optimal Transport library, "
                "JMLR 22(78):1-8, 2021.")
