from .curve_fitting import TimeCurveFitting

__all__ = ["TimeCurveFitting"]
