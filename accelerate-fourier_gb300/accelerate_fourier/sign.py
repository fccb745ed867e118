"""Fourier.Sign (src/Data/Array/Accelerate/Fourier/Sign.hs:28-58):
forward = -1 (time -> frequency), inverse = +1; transforms are unscaled."""
forward = -1
inverse = 1


def check(sign: int) -> int:
    if sign not in (-1, 1):
        raise ValueError("sign must be forward (-1) or inverse (+1)")
    return sign
