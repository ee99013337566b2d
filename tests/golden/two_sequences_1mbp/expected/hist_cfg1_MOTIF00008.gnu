set output "hist_cfg1_MOTIF00008.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-50.5169:14.7526]
set yrange [0:138297]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00008.dat" using 1:2 title 'MOTIF00008 (cfg1)' with boxes
