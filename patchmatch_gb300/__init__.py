"""GB300-native PatchMatch-Stereo densification of equirectangular keyframes."""
