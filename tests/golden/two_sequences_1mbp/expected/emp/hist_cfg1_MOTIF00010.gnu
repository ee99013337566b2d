set output "hist_cfg1_MOTIF00010.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-50.0681:12.2972]
set yrange [0:2175]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00010.dat" using 1:2 title 'MOTIF00010 (cfg1)' with boxes
