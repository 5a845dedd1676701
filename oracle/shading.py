"""Test infrastructure only: restatement of diffren's point-light shader
(diffren/jax/utils/shaders.py:100-173) in torch, any float dtype, for
checking shaded renders and their gradients: light and view directions
l2-normalized (transforms.py:26-37), n.l and n.h clipped to [0, 1], luma
ka + kd n.l + ks (n.h)^ns, attenuation 1 / (c + l d + q d^2)."""
import torch


def _normalize(x):
  return x * torch.rsqrt((x * x).sum(-1, keepdim=True) + 1e-12)


def point_light(diffuse, normals, positions, light, eye=(0.0, 0.0, 0.0), ka=0.3, kd=1.4,
                ks=0.0, ns=0.0, att_c=1.0, att_l=0.7, att_q=1.8):
  light = torch.as_tensor(light, dtype=positions.dtype)
  eye = torch.as_tensor(eye, dtype=positions.dtype)
  ld = _normalize(light - positions)
  vd = _normalize(eye - positions)
  h = _normalize(ld + vd)
  nol = torch.clamp((normals * ld).sum(-1, keepdim=True), 0.0, 1.0)
  noh = torch.clamp((normals * h).sum(-1, keepdim=True), 0.0, 1.0)
  d = torch.sqrt(((light - positions) ** 2).sum(-1, keepdim=True))
  decay = 1.0 / (att_c + att_l * d + att_q * d * d)
  return diffuse * (ka + kd * nol + ks * noh ** ns) * decay
