"""torch.autograd wrapper of the library's convolution and its adjoint
(test harness only; the product is the C ABI).

forward : y = conv3d(image, kernel)                      (fc_conv3d_device)
backward: grad_image  = correlation of grad_y with the kernel
          grad_kernel = correlation of the image with grad_y, cropped to the
                        kernel support                   (fc_conv3d_adjoint_device)
The adjoint recomputes the kernel and image spectra instead of keeping them
from the forward pass, so a large volume costs no extra memory between the
two passes.
"""
import torch

from fourierconvolutioncudalib_gb300 import device as fcd


class FourierConv3d(torch.autograd.Function):
    @staticmethod
    def forward(ctx, image, kernel):
        image = image.contiguous()
        kernel = kernel.contiguous()
        ctx.save_for_backward(image, kernel)
        return fcd.conv3d(image, kernel)

    @staticmethod
    def backward(ctx, grad_out):
        image, kernel = ctx.saved_tensors
        gi, gk = fcd.conv3d_adjoint(image, kernel, grad_out.contiguous(), tuple(kernel.shape),
                                    need_image_grad=ctx.needs_input_grad[0],
                                    need_kernel_grad=ctx.needs_input_grad[1])
        return gi, gk


def fourier_conv3d(image, kernel):
    return FourierConv3d.apply(image, kernel)
