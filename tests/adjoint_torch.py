"""torch.autograd wrapper of the path-replay adjoint, for the tests only.

PathTracedImage.apply(kd, ka, renderer, first_sample, spp) renders samples
[first_sample, first_sample + spp) of every pixel with the given material
albedos / emissions and returns the mean image [H*W, 3]; backward() calls
crt_render_adjoint on the same samples with adjoint = grad_image / spp."""
import numpy as np
import torch


class PathTracedImage(torch.autograd.Function):
    @staticmethod
    def forward(ctx, kd, ka, renderer, first_sample, spp):
        renderer.scene.set_materials(kd.detach().cpu().numpy(), ka.detach().cpu().numpy())
        renderer.restart(first_sample)
        renderer.render(spp)
        img = torch.from_numpy(renderer.accum()).to(kd.device) / spp
        ctx.renderer, ctx.first_sample, ctx.spp = renderer, first_sample, spp
        ctx.n_mats = kd.shape[0]
        return img

    @staticmethod
    def backward(ctx, grad_img):
        r = ctx.renderer
        adj = torch.zeros((grad_img.shape[0], 4), dtype=torch.float32, device="cuda")
        adj[:, :3] = grad_img.to("cuda", torch.float32) / ctx.spp
        gkd = torch.zeros((ctx.n_mats, 3), dtype=torch.float32, device="cuda")
        gka = torch.zeros((ctx.n_mats, 3), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        r.adjoint(ctx.first_sample, ctx.spp, adj.data_ptr(), gkd.data_ptr(), gka.data_ptr())
        r.synchronize()
        return gkd.to(grad_img.device), gka.to(grad_img.device), None, None, None


def material_arrays(sc):
    kd = np.array([m.kd for m in sc.materials], np.float32)
    ka = np.array([m.ka for m in sc.materials], np.float32)
    return kd, ka
