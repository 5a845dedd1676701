"""Image compositing (diffren/jax/composite.py:20-37)."""
import torch


def over(color_layers: torch.Tensor) -> torch.Tensor:
  """'over' compositing of premultiplied [l, h, w, c] layers, layer 0 in front.

  The last channel is alpha. Plain torch ops (differentiable); the splat path
  composites inside its CUDA kernel instead.
  """
  output = color_layers[-1]
  for i in range(2, color_layers.shape[0] + 1):
    alpha = color_layers[-i, ..., -1:]
    output = color_layers[-i] + (1.0 - alpha) * output
  return output
