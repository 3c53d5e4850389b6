"""Gradient-check harness: a torch.autograd.Function around the renderer.

Lives only in the tests.  forward(albedo, strength) renders the image through
the C ABI (wf_scene_set_albedo, wf_scene_set_emission, wf_render);
backward(dL/dimage) calls the path-replay adjoint (wf_adjoint).
"""
import numpy as np
import torch


class RenderImage(torch.autograd.Function):
    @staticmethod
    def forward(ctx, albedo, strength, renderer, light_instance, settings):
        r = renderer
        r.set_albedo(albedo.detach().cpu().numpy())
        r.set_emission(light_instance, float(strength.detach().cpu().item()))
        r.render(max_bounces=settings["max_bounces"], spp=settings["spp"], frame_seed=settings["frame_seed"],
                 nee=settings.get("nee", 0), rr_start_depth=settings.get("rr_start_depth", 0xFFFFFFFF),
                 accumulate=False)
        img = r.read_image()[..., :3].astype(np.float64)
        ctx.renderer, ctx.light, ctx.settings = r, light_instance, settings
        return torch.from_numpy(img)

    @staticmethod
    def backward(ctx, grad_image):
        s = ctx.settings
        ga, ge = ctx.renderer.adjoint(grad_image.detach().cpu().numpy().astype(np.float32),
                                      max_bounces=s["max_bounces"], spp=s["spp"], frame_seed=s["frame_seed"],
                                      nee=s.get("nee", 0), rr_start_depth=s.get("rr_start_depth", 0xFFFFFFFF))
        return (torch.from_numpy(ga.astype(np.float64)), torch.tensor(float(ge[ctx.light]), dtype=torch.float64),
                None, None, None)
