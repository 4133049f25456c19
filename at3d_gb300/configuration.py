"""Numerical parameters (at3d.configuration.get_config, at3d/configuration.py:172,
defaults of default_config.json)."""
from ._abi import NumericalParams


def get_config(**overrides) -> NumericalParams:
    p = NumericalParams()
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    if p.split_accuracy > 0:
        raise ValueError("adaptive cell splitting is not supported: set split_accuracy=0")
    return p
