set output "hist_cfg1_MOTIF00026.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-77.2827:25.7619]
set yrange [0:181959]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00026.dat" using 1:2 title 'MOTIF00026 (cfg1)' with boxes
