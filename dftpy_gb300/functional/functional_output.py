"""FunctionalOutput and its algebra (src/dftpy/functional/functional_output.py:8-126)."""
import copy

__all__ = ["FunctionalOutput", "ZeroFunctional"]

_ATTRS = ["energy", "potential", "energydensity", "v2rho2", "v3rho3", "v4rho4", "force", "stress"]


class FunctionalOutput:
    def __init__(self, name=None, energy=None, potential=None, energydensity=None, v2rho2=None, v3rho3=None,
                 v4rho4=None, force=None, stress=None):
        if name is None:
            raise AttributeError("Functional name must be specified")
        self.name = name
        for k, v in (("energy", energy), ("potential", potential), ("energydensity", energydensity),
                     ("v2rho2", v2rho2), ("v3rho3", v3rho3), ("v4rho4", v4rho4), ("force", force),
                     ("stress", stress)):
            if v is not None:
                setattr(self, k, v)
        self.attr_list = list(_ATTRS)

    def __iter__(self):
        for key in _ATTRS:
            if hasattr(self, key):
                yield key, getattr(self, key)

    def sum(self, other=None):
        if other is None:
            return self.copy()
        name = self.name if self.name == other.name else self.name + other.name
        out = FunctionalOutput(name=name)
        for k, v in self:
            setattr(out, k, v + getattr(other, k) if hasattr(other, k) else v)
        for k, v in other:
            if not hasattr(out, k):
                setattr(out, k, v)
        return out

    def sub(self, other):
        out = self.copy()
        for k, v in self:
            setattr(out, k, v - getattr(other, k) if hasattr(other, k) else v)
        for k, v in other:
            if not hasattr(out, k):
                setattr(out, k, -v)
        return out

    def mul(self, x):
        out = self.copy()
        for k, v in out:
            setattr(out, k, v * x)
        return out

    def div(self, x):
        if x == 0:
            raise ValueError("Dividing zero")
        out = self.copy()
        for k, v in out:
            setattr(out, k, v / x)
        return out

    __add__ = sum
    __sub__ = sub
    __mul__ = mul
    __truediv__ = div

    def __radd__(self, other):
        return self.copy() if other is None or other == 0 else self.sum(other)

    def copy(self):
        out = FunctionalOutput(name=self.name)
        for k, v in self:
            setattr(out, k, v.clone() if hasattr(v, "clone") else copy.deepcopy(v))
        return out

    def __repr__(self):
        return "FunctionalOutput(name=%r, energy=%r)" % (self.name, getattr(self, "energy", None))


class ZeroFunctional:
    """ZeroFunctional (functional_output.py:114-126)."""

    def __call__(self, rho, *args, **kwargs):
        return self.compute(rho, *args, **kwargs)

    @staticmethod
    def compute(rho, *args, calcType={"E", "V"}, **kwargs):
        out = FunctionalOutput(name="ZERO", energy=0.0)
        if "V" in calcType:
            out.potential = rho * 0
        return out
