"""Drop-in for pyaxisymflow/elasto_kernels/extrapolate_using_least_squares.py:8-38."""
import torch

from ..core.extrapolate_using_least_squares import (
    extrapolate_using_least_squares_till_first_order as extrapolate_using_least_squares,
)


def extrapolate_eta_using_least_squares(inp_phi, phi_thresh_lower_bound, phi_thresh_upper_bound,
                                        inp_eta_X, inp_eta_Y, inp_x, inp_y):
    """Extrapolates inp_eta_X, inp_eta_Y from {phi < lower} into {phi < upper}."""
    current_flag = (inp_phi < phi_thresh_lower_bound).to(torch.int16)
    target_flag = (inp_phi < phi_thresh_upper_bound).to(torch.int16)
    extrapolate_using_least_squares(current_flag, target_flag, inp_eta_X, inp_eta_Y, inp_x, inp_y)
